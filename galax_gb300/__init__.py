"""galax_gb300 -- GB300 (sm_103a) FMM force backend for knekvasil/galax.

Python mirror of the reference's GPU backend API (galax-gpu/src/lib.rs:
``GpuConfig``, ``GpuContext::{new, upload_tree_data, step, read_accelerations,
crosscheck, n2_debug}``, ``GpuError``) over the C ABI of ``libgalaxcu.so``
(include/galax_gb300.h).  The library is loaded from ``galax_gb300/_build``;
there is no CPU fallback: without the CUDA library or a GPU every entry point
raises ``GpuError``.
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass, field

import numpy as np

__all__ = [
    "GpuConfig", "GpuContext", "GpuError", "Bodies", "MODE_REF", "MODE_EXACT", "MODE_ACCURATE", "PREC_FP64",
    "PREC_MIXED", "LIST_V", "LIST_U", "lib", "library_path", "HostArray",
]

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgalaxcu.so")

MODE_REF, MODE_EXACT, MODE_ACCURATE = 0, 1, 2
PREC_FP64, PREC_MIXED = 0, 1
LIST_V, LIST_U = 0, 1
BUILD_BALANCED = 1
STATUS_SANITIZED = 1  # gx_last_status: invalid positions / masses were replaced
LIST_CAP = 64

STATUS_NAMES = {
    0: "OK", 1: "InitFailed", 2: "KernelLoad", 3: "BufferAllocation", 4: "InvalidArgument", 5: "NonFinite",
    6: "CapExceeded", 7: "Timeout", 8: "State", 9: "Cuda",
}


class GpuError(RuntimeError):
    """GpuError (galax-gpu/src/lib.rs:42-59) with the C ABI status code."""

    def __init__(self, code: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(code, code)}: {msg}")
        self.code = code


class _Config(C.Structure):
    _fields_ = [("max_n", C.c_uint32), ("max_nodes", C.c_uint32), ("max_interactions", C.c_uint32),
                ("p", C.c_uint32), ("eps", C.c_float), ("eps64", C.c_double), ("device", C.c_int32)]


_lib = None
_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_I32 = C.POINTER(C.c_int32)
_U32 = C.POINTER(C.c_uint32)
_U8 = C.POINTER(C.c_uint8)
_VP = C.c_void_p


def library_path() -> str:
    return _LIB_PATH


def lib():
    """Loads libgalaxcu.so (built by galax_gb300/build.py); raises GpuError if absent."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(_LIB_PATH):
        raise GpuError(2, f"CUDA library not built: {_LIB_PATH} (run galax_gb300/build.py)")
    L = C.CDLL(_LIB_PATH)
    sig = {
        "gx_abi_version": (C.c_int, []),
        "gx_config_default": (C.c_int, [C.POINTER(_Config)]),
        "gx_create": (C.c_int, [C.POINTER(_Config), C.POINTER(_VP)]),
        "gx_destroy": (C.c_int, [_VP]),
        "gx_last_error": (C.c_char_p, [_VP]),
        "gx_set_mode": (C.c_int, [_VP, C.c_int, C.c_int, C.c_double]),
        "gx_set_params": (C.c_int, [_VP, C.c_uint32, C.c_double]),
        "gx_set_near_split": (C.c_int, [_VP, C.c_double]),
        "gx_set_body_split": (C.c_int, [_VP, C.c_double]),
        "gx_plan_body_split_info": (C.c_int, [_VP, _I64, _I64]),
        "gx_plan_split_info": (C.c_int, [_VP, _I64, _I64]),
        "gx_upload_tree": (C.c_int, [_VP, C.c_int64, C.c_int64, _D, _D, _D, _D, _D, _D, _I64, _I64, _I32, _I32, _U8,
                                     _U32, _U8, _U32, _U8]),
        "gx_build_tree": (C.c_int, [_VP, C.c_int64, _D, _D, _D, _D, _D, _D, _D, C.c_int64, _D, C.c_int]),
        "gx_rebuild_resident": (C.c_int, [_VP, C.c_int64, _D, C.c_int, _I64]),
        "gx_tree_info": (C.c_int, [_VP, _I64, _I64, _I32, _I64]),
        "gx_morton_encode": (C.c_int, [_VP, C.c_int64, _D, _D, _D, C.POINTER(C.c_uint64)]),
        "gx_export_tree": (C.c_int, [_VP, _D, _D, _D, _D, _D, _D, _I64, _I64, _I32, _I32, _U8, _I64]),
        "gx_export_lists": (C.c_int, [_VP, C.c_int, _U32, _U8]),
        "gx_plan_info": (C.c_int, [_VP, _I64, _I64, _I64]),
        "gx_compute_forces": (C.c_int, [_VP, _D, _D, _D, _D, _D]),
        "gx_upload_bodies": (C.c_int, [_VP, C.c_int64, _D, _D, _D, _D, _D, _D, _D]),
        "gx_download_bodies": (C.c_int, [_VP, _D, _D, _D, _D, _D, _D, _D]),
        "gx_forces_resident": (C.c_int, [_VP]),
        "gx_kdk_run": (C.c_int, [_VP, C.c_int64, C.c_double, C.c_int64, _D, _I64]),
        "gx_diagnostics": (C.c_int, [_VP, _D]),
        "gx_n2_sampled": (C.c_int, [_VP, _I64, C.c_int64, _D, _D]),
        "gx_last_timings": (C.c_int, [_VP, _D]),
        "gx_bench_forces": (C.c_int, [_VP, C.c_int32, C.c_int32, _D, C.c_int32, _D]),
        "gx_last_launch_count": (C.c_int, [_VP, _I64]),
        "gx_last_status": (C.c_int, [_VP, C.POINTER(C.c_uint32)]),
        "gx_probe_fp32_tflops": (C.c_int, [_VP, _D]),
        "gx_n2_sampled_static": (C.c_int, [_VP, _VP, _VP, C.c_int64, C.c_double, _I64, C.c_int64, _D, _D, _VP]),
        "gx_force_vjp": (C.c_int, [_VP, _D, _D, _D, _D, _D]),
        "gx_rollout_forward": (C.c_int, [_VP, C.c_int64, C.c_double, C.c_int64, C.c_int64]),
        "gx_kdk_run_rebuild": (C.c_int, [_VP, C.c_int64, C.c_double, C.c_int64, C.c_int64, _D, _I64]),
        "gx_body_ids": (C.c_int, [_VP, _I64]),
        "gx_rollout_backward": (C.c_int, [_VP, _D, _D, _D, _D, _D, _D, _D, _D, _D, _I64]),
        "gx_host_alloc": (_VP, [C.c_size_t]),
        "gx_host_free": (None, [_VP]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _p(a, ptype=_D):
    if a is None:
        return None
    return a.ctypes.data_as(ptype)


def _f64(a) -> np.ndarray:
    a = np.asarray(a)
    if a.dtype != np.float64 or not a.flags.c_contiguous:
        raise TypeError("expected a C-contiguous float64 array")
    return a


N2_STATIC_MAX_SAMPLES = 4096


def _mag_rel_err(ax, ay, ex, ey):
    """||a| - |a*|| / max(|a*|, 1e-20) per body (validate_fmm, galax-core/src/lib.rs:1553-1557)."""
    fm = np.sqrt(np.asarray(ax) ** 2 + np.asarray(ay) ** 2)
    em = np.sqrt(np.asarray(ex) ** 2 + np.asarray(ey) ** 2)
    return np.abs(fm - em) / np.maximum(np.abs(em), 1e-20)


def n2_sampled_static(x_dev: int, y_dev: int, m_dev: int, n: int, eps: float, idx, stream: int = 0):
    """Exact FP64 softened forces on sampled targets from the caller's device arrays
    (addresses of n float64 values each), without a context and without allocating
    device memory: for callers that cannot allocate when they want the check (their
    device memory is owned by another runtime's caching allocator).  At most
    N2_STATIC_MAX_SAMPLES targets per call.  `stream` must not be capturing: the call
    copies through pageable host memory and waits for the stream.  The device address
    of the staging array is looked up on the first call on a device and kept for the
    life of the process.  Calls that overlap on the GPU race on the shared staging
    array."""
    idx = np.ascontiguousarray(np.asarray(idx, np.int64))
    ax = np.zeros(idx.size)
    ay = np.zeros(idx.size)
    rc = lib().gx_n2_sampled_static(x_dev, y_dev, m_dev, int(n), float(eps), _p(idx, _I64), idx.size, _p(ax), _p(ay),
                                    stream or None)
    if rc == 6:
        raise GpuError(rc, f"{idx.size} samples exceed the static staging array ({N2_STATIC_MAX_SAMPLES})")
    if rc != 0:
        raise GpuError(rc, "gx_n2_sampled_static failed")
    return ax, ay


class HostArray:
    """A page-locked float64 host buffer (gx_host_alloc) viewed as a numpy array."""

    def __init__(self, n: int):
        self._ptr = lib().gx_host_alloc(max(int(n), 1) * 8)
        if not self._ptr:
            raise GpuError(3, "pinned host allocation failed")
        buf = (C.c_double * max(int(n), 1)).from_address(self._ptr)
        self.array = np.frombuffer(buf, dtype=np.float64, count=int(n))

    def __del__(self):
        try:
            if self._ptr:
                lib().gx_host_free(self._ptr)
                self._ptr = None
        except Exception:
            pass


@dataclass
class Bodies:
    """BodiesSoA (galax-core/src/lib.rs:41-71): seven float64 arrays."""
    x: np.ndarray
    y: np.ndarray
    vx: np.ndarray
    vy: np.ndarray
    mass: np.ndarray
    ax: np.ndarray
    ay: np.ndarray

    @staticmethod
    def new(n: int) -> "Bodies":
        return Bodies(*[np.zeros(n) for _ in range(7)])

    @staticmethod
    def from_arrays(x, y, mass, vx=None, vy=None) -> "Bodies":
        n = len(x)
        z = np.zeros(n)
        f = lambda a: np.ascontiguousarray(np.asarray(a, np.float64)).copy()
        return Bodies(f(x), f(y), f(vx if vx is not None else z), f(vy if vy is not None else z), f(mass), z.copy(),
                      z.copy())

    def __len__(self) -> int:
        return int(self.x.size)

    def copy(self) -> "Bodies":
        return Bodies(*[a.copy() for a in (self.x, self.y, self.vx, self.vy, self.mass, self.ax, self.ay)])


@dataclass
class GpuConfig:
    """GpuConfig (galax-gpu/src/lib.rs:22-40).  ``eps64`` (if > 0) is the FP64 softening."""
    max_n: int = 262_144
    max_nodes: int = 524_288
    max_interactions: int = 1 << 24
    p: int = 4
    eps: float = 0.1
    eps64: float = 0.0
    device: int = 0

    def _c(self) -> _Config:
        return _Config(self.max_n, self.max_nodes, self.max_interactions, self.p, self.eps, self.eps64, self.device)


@dataclass
class DeviceTree:
    """Host copy of a device-built tree (the fields of galax-core's Node, lib.rs:117-129)."""
    cx: np.ndarray
    cy: np.ndarray
    hw: np.ndarray
    mass: np.ndarray
    comx: np.ndarray
    comy: np.ndarray
    body_start: np.ndarray
    body_end: np.ndarray
    child: np.ndarray
    parent: np.ndarray
    is_leaf: np.ndarray
    level_start: np.ndarray
    n_nodes: int = 0
    n_leaves: int = 0
    n_levels: int = 0


class GpuContext:
    """GpuContext (galax-gpu/src/lib.rs:233-714) on libgalaxcu.

    ``GpuContext(config)`` replaces ``GpuContext::new(device, queue, config)``:
    there are no wgpu handles, the CUDA device is ``config.device``.
    """

    def __init__(self, config: GpuConfig | None = None):
        self.config = config or GpuConfig()
        L = lib()
        h = _VP()
        rc = L.gx_create(C.byref(self.config._c()), C.byref(h))
        if rc != 0:
            raise GpuError(rc, "gx_create failed (no CUDA device, or the sm_103a image does not load)")
        self._h = h
        self._ax = None
        self._ay = None

    # -- plumbing
    def _check(self, rc: int) -> None:
        if rc != 0:
            msg = lib().gx_last_error(self._h)
            raise GpuError(rc, msg.decode() if msg else "")

    def close(self) -> None:
        if getattr(self, "_h", None):
            lib().gx_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- configuration
    def set_mode(self, mode: int = MODE_REF, precision: int = PREC_FP64, theta: float = 0.5) -> None:
        self._check(lib().gx_set_mode(self._h, int(mode), int(precision), float(theta)))

    def set_params(self, p: int, eps: float) -> None:
        self._check(lib().gx_set_params(self._h, int(p), float(eps)))

    def set_near_split(self, theta_w: float) -> None:
        """Leaf-level M2P / P2L for near leaf pairs that are far on one side (ACCURATE mode;
        0 turns it off).  The adjoint entry points need it off."""
        self._check(lib().gx_set_near_split(self._h, float(theta_w)))

    def plan_split_info(self):
        """(M2P leaf pairs, P2L leaf pairs) of the current ACCURATE plan."""
        a, b = C.c_int64(), C.c_int64()
        self._check(lib().gx_plan_split_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    def set_body_split(self, theta_b: float) -> None:
        """Body-level P2L of the P2P pairs the near-list split leaves: a source body far
        enough from the target leaf's COM (|x_j - com_a| theta_b > R_a) joins its local
        expansion instead of P2P (needs theta_w > 0 and leaves of at most 32 bodies; 0
        turns it off)."""
        self._check(lib().gx_set_body_split(self._h, float(theta_b)))

    def plan_body_split_info(self):
        """(P2P interactions moved to body-level P2L, body-level P2L evaluations) of the
        current ACCURATE plan."""
        a, b = C.c_int64(), C.c_int64()
        self._check(lib().gx_plan_body_split_info(self._h, C.byref(a), C.byref(b)))
        return a.value, b.value

    # -- trees
    def upload_tree_data(self, tree, m2l_lists, p2p_lists) -> None:
        """upload_tree_data (galax-gpu/src/lib.rs:392-462): a host tree + V/U lists in the reference layout."""
        n = int(tree.n_nodes)
        nb = int(tree.body_end.max()) if n else 0
        f = lambda a, dt: np.ascontiguousarray(np.asarray(a, dt))
        arrs = [f(tree.cx, np.float64), f(tree.cy, np.float64), f(tree.hw, np.float64), f(tree.mass, np.float64),
                f(tree.comx, np.float64), f(tree.comy, np.float64)]
        bs, be = f(tree.body_start, np.int64), f(tree.body_end, np.int64)
        ch, par, leaf = f(tree.child, np.int32), f(tree.parent, np.int32), f(tree.is_leaf, np.uint8)
        vd, vl = f(m2l_lists.data, np.uint32), f(m2l_lists.lengths, np.uint8)
        ud, ul = f(p2p_lists.data, np.uint32), f(p2p_lists.lengths, np.uint8)
        self._check(lib().gx_upload_tree(self._h, n, nb, *[_p(a) for a in arrs], _p(bs, _I64), _p(be, _I64),
                                         _p(ch, _I32), _p(par, _I32), _p(leaf, _U8), _p(vd, _U32), _p(vl, _U8),
                                         _p(ud, _U32), _p(ul, _U8)))

    def build_tree(self, bodies: Bodies, n_max: int, bounds, balanced: bool = False) -> None:
        """Device Tree::build (or build_constrained); permutes ``bodies`` in place like the reference."""
        b = np.ascontiguousarray(np.asarray(bounds, np.float64))
        arrs = [_f64(a) for a in (bodies.x, bodies.y, bodies.vx, bodies.vy, bodies.mass, bodies.ax, bodies.ay)]
        self._check(lib().gx_build_tree(self._h, len(bodies), *[_p(a) for a in arrs], int(n_max), _p(b),
                                        BUILD_BALANCED if balanced else 0))
        self._n_resident = len(bodies)

    def rebuild_resident(self, n_max: int, bounds, balanced: bool = False, want_perm: bool = False):
        """Tree::build over the resident bodies (they are permuted on the device); returns,
        if asked, each body's index before the rebuild."""
        b = np.ascontiguousarray(np.asarray(bounds, np.float64))
        n = getattr(self, "_n_resident", 0)
        perm = np.zeros(n, np.int64) if (want_perm and n > 0) else None
        self._check(lib().gx_rebuild_resident(self._h, int(n_max), _p(b), BUILD_BALANCED if balanced else 0,
                                              _p(perm, _I64) if perm is not None else None))
        return perm

    def morton_encode(self, x, y, bounds) -> np.ndarray:
        """morton_encode (galax-core/src/lib.rs:95-109) of many bodies on the device."""
        x = np.ascontiguousarray(np.asarray(x, np.float64))
        y = np.ascontiguousarray(np.asarray(y, np.float64))
        b = np.ascontiguousarray(np.asarray(bounds, np.float64))
        keys = np.zeros(x.size, np.uint64)
        self._check(lib().gx_morton_encode(self._h, x.size, _p(x), _p(y), _p(b),
                                           keys.ctypes.data_as(C.POINTER(C.c_uint64))))
        return keys

    def tree_info(self):
        nn, nl, nb = C.c_int64(), C.c_int64(), C.c_int64()
        lv = C.c_int32()
        self._check(lib().gx_tree_info(self._h, C.byref(nn), C.byref(nl), C.byref(lv), C.byref(nb)))
        return nn.value, nl.value, lv.value, nb.value

    def export_tree(self) -> DeviceTree:
        nn, nl, lv, _ = self.tree_info()
        t = DeviceTree(*[np.zeros(nn) for _ in range(6)], np.zeros(nn, np.int64), np.zeros(nn, np.int64),
                       np.zeros((nn, 4), np.int32), np.zeros(nn, np.int32), np.zeros(nn, np.uint8),
                       np.zeros(lv + 1, np.int64), nn, nl, lv)
        self._check(lib().gx_export_tree(self._h, _p(t.cx), _p(t.cy), _p(t.hw), _p(t.mass), _p(t.comx), _p(t.comy),
                                         _p(t.body_start, _I64), _p(t.body_end, _I64), _p(t.child, _I32),
                                         _p(t.parent, _I32), _p(t.is_leaf, _U8), _p(t.level_start, _I64)))
        return t

    def export_lists(self, which: int):
        nn = self.tree_info()[0]
        data = np.zeros((nn, LIST_CAP), np.uint32)
        lengths = np.zeros(nn, np.uint8)
        self._check(lib().gx_export_lists(self._h, int(which), _p(data, _U32), _p(lengths, _U8)))
        return data, lengths

    def plan_info(self):
        a, b, c = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(lib().gx_plan_info(self._h, C.byref(a), C.byref(b), C.byref(c)))
        return a.value, b.value, c.value

    # -- forces
    def step(self, bodies: Bodies) -> None:
        """step (galax-gpu/src/lib.rs:464-544): uploads x, y, mass and runs the six passes."""
        n = len(bodies)
        self._ax = np.zeros(n)
        self._ay = np.zeros(n)
        self._check(lib().gx_compute_forces(self._h, _p(_f64(bodies.x)), _p(_f64(bodies.y)), _p(_f64(bodies.mass)),
                                            _p(self._ax), _p(self._ay)))

    def read_accelerations(self, ax: np.ndarray, ay: np.ndarray) -> None:
        """read_accelerations (galax-gpu/src/lib.rs:546-566)."""
        if self._ax is None:
            raise GpuError(8, "read_accelerations before step")
        n = min(ax.size, ay.size, self._ax.size)
        ax[:n] = self._ax[:n]
        ay[:n] = self._ay[:n]

    def compute_forces(self, x, y, m, ax, ay) -> None:
        """One call: host x, y, m in; host ax, ay out (C ABI gx_compute_forces)."""
        self._check(lib().gx_compute_forces(self._h, _p(_f64(x)), _p(_f64(y)), _p(_f64(m)), _p(_f64(ax)),
                                            _p(_f64(ay))))

    def crosscheck(self, bodies: Bodies, cpu_ax: np.ndarray, cpu_ay: np.ndarray, threshold: float):
        """crosscheck (galax-gpu/src/lib.rs:628-667) against caller-supplied CPU accelerations:
        per-body |da| / max(|a_cpu|, |a_gpu|, 1e-30); raises above ``threshold``."""
        self.step(bodies)
        gx, gy = self._ax, self._ay
        cm = np.hypot(cpu_ax, cpu_ay)
        gm = np.hypot(gx, gy)
        den = np.maximum(np.maximum(cm, gm), 1e-30)
        rel = np.hypot(gx - cpu_ax, gy - cpu_ay) / den
        mx, mean = float(rel.max()) if rel.size else 0.0, float(rel.mean()) if rel.size else 0.0
        if mx > threshold:
            raise GpuError(0, f"GPU crosscheck max relative error {mx:.2e} exceeds threshold {threshold:.2e}")
        return mx, mean, rel.size

    def validate_fmm(self, bodies: Bodies, sample_size: int, seed: int = 0):
        """validate_fmm (galax-core/src/lib.rs:1502-1564): the FMM of the context's mode and
        precision on all bodies, the exact FP64 softened sum (GPU) on ``sample_size`` bodies
        drawn without replacement, and the magnitude error ||a| - |a*|| / max(|a*|, 1e-20)
        of each.  Returns (sample_size, max, mean, 0.0) as the reference does.  The draw is
        seeded here (the reference shuffles with an unseeded generator).  ``bodies`` must be
        in the order the context's tree was built on; they become the resident bodies."""
        n = len(bodies)
        k = min(int(sample_size), n)
        self.upload_bodies(bodies)
        self.forces_resident()
        out = Bodies.new(n)
        self.download_bodies(out)
        idx = np.sort(np.random.default_rng(seed).permutation(n)[:k]).astype(np.int64)
        ex, ey = self.n2_sampled(idx)
        rel = _mag_rel_err(out.ax[idx], out.ay[idx], ex, ey)
        mean = float(rel.sum()) / k if k else float("nan")  # the reference divides by sample_size
        return k, float(rel.max()) if k else 0.0, mean, 0.0

    def n2_regression(self, bodies: Bodies) -> float:
        """n2_regression (galax-core/src/lib.rs:1567-1598): the FMM against the exact FP64 sum
        on every body (N <= 2000), largest magnitude error.  ``bodies`` as for validate_fmm."""
        n = len(bodies)
        if n > 2000:
            raise ValueError("n2_regression only valid for N <= 2000")
        self.upload_bodies(bodies)
        self.forces_resident()
        out = Bodies.new(n)
        self.download_bodies(out)
        ex, ey = self.n2_sampled(np.arange(n, dtype=np.int64))
        rel = _mag_rel_err(out.ax, out.ay, ex, ey)
        return float(rel.max()) if n else 0.0

    def n2_debug(self, bodies: Bodies):
        """n2_debug (galax-gpu/src/lib.rs:670-714): exact FP64 softened forces for every body."""
        self.upload_bodies(bodies)
        return self.n2_sampled(np.arange(len(bodies), dtype=np.int64))

    def convergence(self, bodies: Bodies, n_max: int, bounds, eps: float, orders=(2, 4, 6, 8),
                    sample_size: int = 1000, seed: int = 0):
        """galax-cli --convergence (galax-cli/src/main.rs:355-377): copies of the bodies'
        positions and masses (zero velocities and accelerations, like the CLI's ref_bodies),
        build_constrained on them as they are ordered (it does not sort;
        galax-core/src/lib.rs:541-588), the reference's V/U lists of that tree, then
        validate_fmm in REF semantics, FP64, at every order p.  Returns rows
        (p, samples, max, mean) of the magnitude error against the exact sum, the CLI's
        table.  The sample draw is seeded (the reference's is not).  The context is left
        with the balanced tree, REF mode, FP64 and the last order."""
        rb = Bodies.from_arrays(bodies.x, bodies.y, bodies.mass)
        self.build_tree(rb, n_max, bounds, balanced=True)
        self.set_mode(MODE_REF, PREC_FP64, 0.5)
        rows = []
        for p in orders:
            self.set_params(int(p), float(eps))
            k, mx, mean, _ = self.validate_fmm(rb, sample_size, seed)
            rows.append((int(p), k, mx, mean))
        return rows

    # -- resident state
    def upload_bodies(self, b: Bodies) -> None:
        arrs = [_f64(a) for a in (b.x, b.y, b.vx, b.vy, b.mass, b.ax, b.ay)]
        self._check(lib().gx_upload_bodies(self._h, len(b), *[_p(a) for a in arrs]))
        self._n_resident = len(b)

    def download_bodies(self, b: Bodies) -> None:
        arrs = [_f64(a) for a in (b.x, b.y, b.vx, b.vy, b.mass, b.ax, b.ay)]
        self._check(lib().gx_download_bodies(self._h, *[_p(a) for a in arrs]))

    def forces_resident(self) -> None:
        self._check(lib().gx_forces_resident(self._h))

    def kdk_run(self, n_steps: int, dt: float, energy_every: int = 0, rebuild_every: int = 0) -> np.ndarray:
        """Device-resident leapfrog; rebuild_every > 0 rebuilds the tree every that many steps."""
        rows = n_steps // energy_every if energy_every > 0 else 0
        diag = np.zeros(6 * max(rows, 1))
        nd = C.c_int64()
        self._check(lib().gx_kdk_run_rebuild(self._h, int(n_steps), float(dt), int(energy_every), int(rebuild_every),
                                             _p(diag), C.byref(nd)))
        return diag[: 6 * nd.value].reshape(nd.value, 6)

    def simulate(self, n_steps: int, dt: float, energy_every: int = 0, snap_every: int = 0, snapshot=None,
                 rebuild_every: int = 0) -> np.ndarray:
        """simulate (galax-integrate/src/lib.rs:204-237) on the resident bodies, with the
        snapshots the reference CLI's --snap-every asks for (galax-cli/src/main.rs:49):
        every snap_every steps the bodies are read back, in the order of the last upload
        even when the tree is rebuilt, and passed to snapshot(step, bodies) -- e.g. a
        function that writes galx_io.write_snapshot to a file per step.  Returns the
        diagnostics rows of gx_kdk_run (step, KE, FMM PE, px, py, Lz), taken every
        energy_every steps counted from the start of each snapshot interval (from the
        start of the run when snap_every is a multiple of energy_every)."""
        rows = []
        done = 0
        chunk = snap_every if (snap_every > 0 and snapshot is not None) else n_steps
        while done < n_steps:
            k = min(chunk, n_steps - done)
            d = self.kdk_run(k, dt, energy_every, rebuild_every=rebuild_every)
            if d.size:
                d = d.copy()
                d[:, 0] += done
                rows.append(d)
            done += k
            if snapshot is not None and snap_every > 0 and done % snap_every == 0:
                n = getattr(self, "_n_resident", 0)
                out = Bodies.new(n)
                self.download_bodies(out)
                if rebuild_every > 0:  # back to the order of the last upload
                    ids = self.body_ids()
                    for name in ("x", "y", "vx", "vy", "mass", "ax", "ay"):
                        arr = getattr(out, name)
                        res = np.empty_like(arr)
                        res[ids] = arr
                        setattr(out, name, res)
                snapshot(done, out)
        return np.concatenate(rows) if rows else np.zeros((0, 6))

    def diagnostics(self) -> np.ndarray:
        out = np.zeros(5)
        self._check(lib().gx_diagnostics(self._h, _p(out)))
        return out

    def n2_sampled(self, idx):
        idx = np.ascontiguousarray(np.asarray(idx, np.int64))
        ax = np.zeros(idx.size)
        ay = np.zeros(idx.size)
        self._check(lib().gx_n2_sampled(self._h, _p(idx, _I64), idx.size, _p(ax), _p(ay)))
        return ax, ay

    def last_timings(self) -> np.ndarray:
        out = np.zeros(7)
        self._check(lib().gx_last_timings(self._h, _p(out)))
        return out

    def last_launch_count(self) -> int:
        c = C.c_int64()
        self._check(lib().gx_last_launch_count(self._h, C.byref(c)))
        return c.value

    def last_status(self) -> int:
        """Status bits of the last force evaluation (STATUS_SANITIZED: inputs were sanitised
        as compute_fmm_force does, galax-core/src/lib.rs:1474-1482)."""
        s = C.c_uint32()
        self._check(lib().gx_last_status(self._h, C.byref(s)))
        return s.value

    # -- reverse mode (ACCURATE)
    def _resident_n(self, *arrays) -> int:
        """The resident body count; every cotangent array must have that length."""
        n = self.tree_info()[3]
        for a in arrays:
            if len(a) != n:
                raise ValueError(f"cotangent of length {len(a)} for {n} resident bodies")
        return n

    def force_vjp(self, lam_x, lam_y):
        """(g_x, g_y, g_m) = lam . d(a)/d(x, y, m) at the resident bodies."""
        n = self._resident_n(lam_x, lam_y)
        gx, gy, gm = np.zeros(n), np.zeros(n), np.zeros(n)
        self._check(lib().gx_force_vjp(self._h, _p(_f64(np.ascontiguousarray(lam_x, np.float64))),
                                       _p(_f64(np.ascontiguousarray(lam_y, np.float64))), _p(gx), _p(gy), _p(gm)))
        return gx, gy, gm

    def rollout_forward(self, n_steps: int, dt: float, checkpoint_every: int, rebuild_every: int = 0) -> None:
        self._check(lib().gx_rollout_forward(self._h, int(n_steps), float(dt), int(checkpoint_every),
                                             int(rebuild_every)))

    def body_ids(self) -> np.ndarray:
        """For every resident body, its index in the order of the last upload / build_tree
        (device rebuilds reorder the bodies)."""
        ids = np.zeros(getattr(self, "_n_resident", 0), np.int64)
        if ids.size:
            self._check(lib().gx_body_ids(self._h, _p(ids, _I64)))
        return ids

    def rollout_backward(self, lx, ly, lvx, lvy):
        """Gradients at step 0: (g_x, g_y, g_vx, g_vy, g_m, peak_device_bytes)."""
        n = self._resident_n(lx, ly, lvx, lvy)
        out = [np.zeros(n) for _ in range(5)]
        pk = C.c_int64()
        f = lambda a: _p(_f64(np.ascontiguousarray(a, np.float64)))
        self._check(lib().gx_rollout_backward(self._h, f(lx), f(ly), f(lvx), f(lvy), *[_p(o) for o in out],
                                              C.byref(pk)))
        return (*out, pk.value)

    def probe_fp32_tflops(self) -> float:
        out = C.c_double()
        self._check(lib().gx_probe_fp32_tflops(self._h, C.byref(out)))
        return out.value

    def bench_forces(self, reps: int, flush_l2: bool = True, which: int = 0):
        ms = np.zeros(reps)
        kms = np.zeros(reps)
        self._check(lib().gx_bench_forces(self._h, int(reps), int(flush_l2), _p(ms), int(which), _p(kms)))
        return ms, kms
