"""ctypes wrapper of the CPU oracle (oracle/galax_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and
``bench.py``'s cpu_baseline / ``--impl reference`` leg, never by the product
package.  It restates knekvasil/galax galax-core (Rust) on the CPU; see the
citations in galax_oracle.c.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libgalax_oracle.so")
_lib = None

LIST_CAP = 64
LIST_EMPTY = 0xFFFFFFFF


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP, -ffp-contract=off)."""
    src = os.path.join(_HERE, "galax_oracle.c")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class _Tree(C.Structure):
    _fields_ = [
        ("n_nodes", C.c_int64), ("cap", C.c_int64),
        ("cx", C.POINTER(C.c_double)), ("cy", C.POINTER(C.c_double)), ("hw", C.POINTER(C.c_double)),
        ("mass", C.POINTER(C.c_double)), ("comx", C.POINTER(C.c_double)), ("comy", C.POINTER(C.c_double)),
        ("body_start", C.POINTER(C.c_int64)), ("body_end", C.POINTER(C.c_int64)),
        ("child", C.POINTER(C.c_int32)), ("parent", C.POINTER(C.c_int32)), ("is_leaf", C.POINTER(C.c_uint8)),
        ("n_levels", C.c_int32), ("level_start", C.POINTER(C.c_int64)),
        ("n_max", C.c_int64), ("xmin", C.c_double), ("xmax", C.c_double), ("ymin", C.c_double),
        ("ymax", C.c_double),
    ]


class _Lists(C.Structure):
    _fields_ = [("n_nodes", C.c_int64), ("data", C.POINTER(C.c_uint32)), ("lengths", C.POINTER(C.c_uint8))]


_D = C.POINTER(C.c_double)
_I64 = C.POINTER(C.c_int64)
_TP = C.POINTER(_Tree)
_LP = C.POINTER(_Lists)


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(_LIB_PATH)
        L.gxo_morton_encode.restype = C.c_uint64
        L.gxo_morton_encode.argtypes = [C.c_double] * 6
        L.gxo_morton_decode.argtypes = [C.c_uint64] + [C.c_double] * 4 + [_D, _D]
        L.gxo_morton_encode_many.argtypes = [_D, _D, C.c_int64] + [C.c_double] * 4 + [C.POINTER(C.c_uint64)]
        L.gxo_tree_build.restype = _TP
        L.gxo_tree_build.argtypes = [_D] * 7 + [C.c_int64, C.c_int64] + [C.c_double] * 4
        L.gxo_tree_build_with_constraints.restype = _TP
        L.gxo_tree_build_with_constraints.argtypes = [_D, _D, _D, C.c_int64, C.c_int64] + [C.c_double] * 4 + [_I64, C.c_int64]
        L.gxo_tree_build_constrained.restype = _TP
        L.gxo_tree_build_constrained.argtypes = [_D, _D, _D, C.c_int64, C.c_int64] + [C.c_double] * 4 + [C.c_int]
        L.gxo_tree_free.argtypes = [_TP]
        L.gxo_neighbors_geometric.argtypes = [_TP, C.c_int32, C.POINTER(C.c_int32)]
        L.gxo_compute_levels.argtypes = [_TP, C.POINTER(C.c_uint32)]
        L.gxo_vlist_build.restype = _LP
        L.gxo_vlist_build.argtypes = [_TP, C.c_int]
        L.gxo_ulist_build.restype = _LP
        L.gxo_ulist_build.argtypes = [_TP, C.c_int]
        L.gxo_lists_free.argtypes = [_LP]
        L.gxo_num_moments.restype = C.c_int64
        L.gxo_num_moments.argtypes = [C.c_int64]
        L.gxo_moment_index.restype = C.c_int64
        L.gxo_moment_index.argtypes = [C.c_int64, C.c_int64]
        L.gxo_p2m.argtypes = [_D, _D, _D, _TP, C.c_int64, _D]
        L.gxo_m2m.argtypes = [_D, _TP, C.c_int64]
        L.gxo_kernel_derivs.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int64, _D]
        L.gxo_kernel_derivs_recurrence.argtypes = [C.c_double, C.c_double, C.c_double, C.c_int64, _D]
        L.gxo_m2l.argtypes = [_D, _D, _LP, _TP, C.c_int64, C.c_double, C.c_int]
        L.gxo_m2l_ref_keys.restype = C.c_int64
        L.gxo_m2l_ref_keys.argtypes = [_LP, _TP, C.POINTER(C.c_int32), _D, C.c_int64]
        L.gxo_l2l.argtypes = [_D, _TP, C.c_int64, C.c_int]
        L.gxo_l2p.argtypes = [_D, _D, _D, _D, _D, _TP, C.c_int64]
        L.gxo_p2p.argtypes = [_D, _D, _D, _D, _D, _TP, _LP, C.c_double]
        L.gxo_compute_fmm_force.argtypes = [_D] * 5 + [_TP, _LP, _LP, C.c_int64, C.c_double, C.c_int]
        L.gxo_n2_force.argtypes = [_D, _D, _D, C.c_int64, C.c_double, _D, _D]
        L.gxo_n2_sampled.argtypes = [_D, _D, _D, C.c_int64, C.c_double, _I64, C.c_int64, _D, _D]
        L.gxo_kinetic_energy.restype = C.c_double
        L.gxo_kinetic_energy.argtypes = [_D, _D, _D, C.c_int64]
        L.gxo_momentum.argtypes = [_D, _D, _D, C.c_int64, _D, _D]
        L.gxo_angular_momentum.restype = C.c_double
        L.gxo_angular_momentum.argtypes = [_D] * 5 + [C.c_int64]
        L.gxo_fmm_potential_energy.restype = C.c_double
        L.gxo_fmm_potential_energy.argtypes = [_D] * 5 + [C.c_int64]
        L.gxo_simulate.restype = C.c_int64
        L.gxo_simulate.argtypes = [_D] * 7 + [_TP, _LP, _LP, C.c_int64, C.c_double, C.c_double, C.c_int64,
                                              C.c_int64, C.c_int, _D]
        L.gxo_cli_softening.restype = C.c_double
        L.gxo_cli_softening.argtypes = [_D, _D, C.c_int64]
        L.gxo_set_threads.argtypes = [C.c_int]
        L.gxo_get_threads.restype = C.c_int
        _lib = L
    return _lib


def _d(a: np.ndarray):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(_D)


def _arr(a, dtype=np.float64):
    return np.ascontiguousarray(np.asarray(a, dtype=dtype))


def set_threads(n: int) -> None:
    lib().gxo_set_threads(int(n))


def get_threads() -> int:
    return int(lib().gxo_get_threads())


# ------------------------------------------------------------------ morton
def morton_encode(x, y, xmin, xmax, ymin, ymax) -> int:
    return int(lib().gxo_morton_encode(float(x), float(y), xmin, xmax, ymin, ymax))


def morton_encode_many(x, y, bounds) -> np.ndarray:
    x, y = _arr(x), _arr(y)
    out = np.empty(x.size, np.uint64)
    lib().gxo_morton_encode_many(_d(x), _d(y), x.size, *bounds, out.ctypes.data_as(C.POINTER(C.c_uint64)))
    return out


def morton_decode(key, xmin, xmax, ymin, ymax):
    a, b = C.c_double(), C.c_double()
    lib().gxo_morton_decode(int(key), xmin, xmax, ymin, ymax, C.byref(a), C.byref(b))
    return a.value, b.value


# ------------------------------------------------------------------ bodies
@dataclass
class Bodies:
    """BodiesSoA (galax-core/src/lib.rs:41-71)."""
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
        return Bodies(_arr(x).copy(), _arr(y).copy(), _arr(vx if vx is not None else z).copy(),
                      _arr(vy if vy is not None else z).copy(), _arr(mass).copy(), z.copy(), z.copy())

    def __len__(self):
        return self.x.size

    def copy(self) -> "Bodies":
        return Bodies(*[a.copy() for a in (self.x, self.y, self.vx, self.vy, self.mass, self.ax, self.ay)])


# ------------------------------------------------------------------ tree
class Tree:
    """Owning handle of an oracle tree, with numpy copies of every node field."""

    def __init__(self, ptr):
        self._p = ptr
        t = ptr.contents
        n = t.n_nodes
        self.n_nodes = int(n)

        def cp(pp, count, dt):
            if count == 0:
                return np.zeros(0, dt)
            return np.ctypeslib.as_array(pp, shape=(count,)).astype(dt, copy=True)

        self.cx = cp(t.cx, n, np.float64)
        self.cy = cp(t.cy, n, np.float64)
        self.hw = cp(t.hw, n, np.float64)
        self.mass = cp(t.mass, n, np.float64)
        self.comx = cp(t.comx, n, np.float64)
        self.comy = cp(t.comy, n, np.float64)
        self.body_start = cp(t.body_start, n, np.int64)
        self.body_end = cp(t.body_end, n, np.int64)
        self.child = cp(t.child, 4 * n, np.int32).reshape(n, 4)
        self.parent = cp(t.parent, n, np.int32)
        self.is_leaf = cp(t.is_leaf, n, np.uint8)
        self.n_levels = int(t.n_levels)
        self.level_start = cp(t.level_start, self.n_levels + 1, np.int64) if n else np.zeros(1, np.int64)
        self.n_max = int(t.n_max)
        self.bounds = (t.xmin, t.xmax, t.ymin, t.ymax)

    def __del__(self):
        try:
            if self._p:
                lib().gxo_tree_free(self._p)
        except Exception:
            pass

    @property
    def ptr(self):
        return self._p

    @property
    def n_leaves(self) -> int:
        return int(self.level_start[1]) if self.n_nodes else 0

    def levels(self) -> np.ndarray:
        out = np.zeros(self.n_nodes, np.uint32)
        lib().gxo_compute_levels(self._p, out.ctypes.data_as(C.POINTER(C.c_uint32)))
        return out

    def neighbors_geometric(self, node: int) -> np.ndarray:
        out = np.zeros(8, np.int32)
        lib().gxo_neighbors_geometric(self._p, int(node), out.ctypes.data_as(C.POINTER(C.c_int32)))
        return out


def tree_build(b: Bodies, n_max: int, bounds) -> Tree:
    """Tree::build: permutes ``b`` in place (stable Morton sort)."""
    n = len(b)
    p = lib().gxo_tree_build(_d(b.x), _d(b.y), _d(b.vx), _d(b.vy), _d(b.mass), _d(b.ax), _d(b.ay), n, int(n_max),
                             *map(float, bounds))
    return Tree(p)


def tree_build_with_constraints(b: Bodies, n_max: int, bounds, splits) -> Tree:
    s = np.ascontiguousarray(np.sort(np.asarray(splits, np.int64)))
    p = lib().gxo_tree_build_with_constraints(_d(b.x), _d(b.y), _d(b.mass), len(b), int(n_max), *map(float, bounds),
                                              s.ctypes.data_as(_I64), s.size)
    return Tree(p)


def tree_build_constrained(b: Bodies, n_max: int, bounds, accel: bool = True) -> Tree:
    p = lib().gxo_tree_build_constrained(_d(b.x), _d(b.y), _d(b.mass), len(b), int(n_max), *map(float, bounds),
                                         int(accel))
    return Tree(p)


# ------------------------------------------------------------------ lists
class Lists:
    """InteractionLists (lib.rs:941-944): data (n_nodes, 64) u32, lengths u8."""

    def __init__(self, ptr):
        self._p = ptr
        l = ptr.contents
        n = int(l.n_nodes)
        self.n_nodes = n
        if n:
            self.data = np.ctypeslib.as_array(l.data, shape=(n * LIST_CAP,)).reshape(n, LIST_CAP).copy()
            self.lengths = np.ctypeslib.as_array(l.lengths, shape=(n,)).copy()
        else:
            self.data = np.zeros((0, LIST_CAP), np.uint32)
            self.lengths = np.zeros(0, np.uint8)

    def __del__(self):
        try:
            if self._p:
                lib().gxo_lists_free(self._p)
        except Exception:
            pass

    @property
    def ptr(self):
        return self._p

    def csr(self):
        """(offsets[n+1] u32, indices u32) in node order -- compact_interaction_lists."""
        off = np.zeros(self.n_nodes + 1, np.int64)
        np.cumsum(self.lengths.astype(np.int64), out=off[1:])
        mask = np.arange(LIST_CAP)[None, :] < self.lengths[:, None]
        return off, self.data[mask].astype(np.uint32)


def vlist_build(t: Tree, accel: bool = True) -> Lists:
    return Lists(lib().gxo_vlist_build(t.ptr, int(accel)))


def ulist_build(t: Tree, accel: bool = True) -> Lists:
    return Lists(lib().gxo_ulist_build(t.ptr, int(accel)))


# ------------------------------------------------------------------ passes
def num_moments(p: int) -> int:
    return (p + 1) * (p + 2) // 2


def moment_index(i: int, j: int) -> int:
    n = i + j
    return n * (n + 1) // 2 + j


def kernel_deriv_idx(k: int, l: int, p: int) -> int:
    return (k + l) * (2 * p + 1) + l


def p2m(b: Bodies, t: Tree, p: int) -> np.ndarray:
    out = np.zeros(t.n_nodes * num_moments(p))
    lib().gxo_p2m(_d(b.x), _d(b.y), _d(b.mass), t.ptr, p, _d(out))
    return out


def m2m(mult: np.ndarray, t: Tree, p: int) -> None:
    lib().gxo_m2m(_d(mult), t.ptr, p)


def kernel_derivs(dx, dy, eps, p, recurrence=False) -> np.ndarray:
    out = np.zeros((2 * p + 1) ** 2)
    f = lib().gxo_kernel_derivs_recurrence if recurrence else lib().gxo_kernel_derivs
    f(float(dx), float(dy), float(eps), int(p), _d(out))
    return out


def m2l(locals_: np.ndarray, mult: np.ndarray, v: Lists, t: Tree, p: int, eps: float, mode: int = 0) -> None:
    lib().gxo_m2l(_d(locals_), _d(mult), v.ptr, t.ptr, p, float(eps), int(mode))


def m2l_ref_keys(v: Lists, t: Tree):
    n_pairs = int(v.lengths.astype(np.int64).sum())
    pk = np.zeros(max(n_pairs, 1), np.int32)
    nk = lib().gxo_m2l_ref_keys(v.ptr, t.ptr, pk.ctypes.data_as(C.POINTER(C.c_int32)), None, 0)
    kd = np.zeros(2 * max(nk, 1))
    lib().gxo_m2l_ref_keys(v.ptr, t.ptr, pk.ctypes.data_as(C.POINTER(C.c_int32)), _d(kd), nk)
    return pk[:n_pairs], kd[: 2 * nk].reshape(nk, 2)


def l2l(locals_: np.ndarray, t: Tree, p: int, order: int = 0) -> None:
    lib().gxo_l2l(_d(locals_), t.ptr, p, int(order))


def l2p(b: Bodies, locals_: np.ndarray, t: Tree, p: int) -> None:
    lib().gxo_l2p(_d(b.x), _d(b.y), _d(b.ax), _d(b.ay), _d(locals_), t.ptr, p)


def p2p(b: Bodies, t: Tree, u: Lists, eps: float) -> None:
    lib().gxo_p2p(_d(b.x), _d(b.y), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, u.ptr, float(eps))


MODE_REF = 0
MODE_EXACT = 1


def compute_fmm_force(b: Bodies, t: Tree, v: Lists, u: Lists, p: int, eps: float, mode: int = MODE_REF) -> None:
    """compute_fmm_force (lib.rs:1466-1499): sanitises b in place, fills b.ax/b.ay."""
    lib().gxo_compute_fmm_force(_d(b.x), _d(b.y), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, v.ptr, u.ptr, int(p),
                                float(eps), int(mode))


def n2_force(b: Bodies, eps: float) -> None:
    lib().gxo_n2_force(_d(b.x), _d(b.y), _d(b.mass), len(b), float(eps), _d(b.ax), _d(b.ay))


def n2_sampled(x, y, m, eps, idx):
    x, y, m = _arr(x), _arr(y), _arr(m)
    idx = np.ascontiguousarray(np.asarray(idx, np.int64))
    ax = np.zeros(idx.size)
    ay = np.zeros(idx.size)
    lib().gxo_n2_sampled(_d(x), _d(y), _d(m), x.size, float(eps), idx.ctypes.data_as(_I64), idx.size, _d(ax), _d(ay))
    return ax, ay


def kinetic_energy(b: Bodies) -> float:
    return lib().gxo_kinetic_energy(_d(b.mass), _d(b.vx), _d(b.vy), len(b))


def momentum(b: Bodies):
    px, py = C.c_double(), C.c_double()
    lib().gxo_momentum(_d(b.mass), _d(b.vx), _d(b.vy), len(b), C.byref(px), C.byref(py))
    return px.value, py.value


def angular_momentum(b: Bodies) -> float:
    return lib().gxo_angular_momentum(_d(b.mass), _d(b.x), _d(b.y), _d(b.vx), _d(b.vy), len(b))


def fmm_potential_energy(b: Bodies) -> float:
    return lib().gxo_fmm_potential_energy(_d(b.mass), _d(b.x), _d(b.y), _d(b.ax), _d(b.ay), len(b))


def simulate(b: Bodies, t: Tree, v: Lists, u: Lists, p: int, eps: float, dt: float, n_steps: int,
             energy_every: int, mode: int = MODE_REF) -> np.ndarray:
    nd = n_steps // energy_every if energy_every > 0 else 0
    diag = np.zeros(6 * max(nd, 1))
    k = lib().gxo_simulate(_d(b.x), _d(b.y), _d(b.vx), _d(b.vy), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, v.ptr, u.ptr,
                           int(p), float(eps), float(dt), int(n_steps), int(energy_every), int(mode), _d(diag))
    return diag[: 6 * k].reshape(k, 6)


def cli_softening(b: Bodies) -> float:
    return lib().gxo_cli_softening(_d(b.x), _d(b.y), len(b))


def cli_dt(ax: np.ndarray, ay: np.ndarray) -> float:
    """dt = 0.5/sqrt(max|a|) else 0.01 (galax-cli/src/main.rs:232-244); the fold over
    f64::max ignores NaN."""
    a = np.sqrt(np.asarray(ax) * np.asarray(ax) + np.asarray(ay) * np.asarray(ay))
    amax = float(np.nanmax(np.concatenate([a, [0.0]])))
    return 0.5 / amax ** 0.5 if amax > 1e-30 else 0.01


# ------------------------------------------------------------ accurate mode
class _Csr(C.Structure):
    _fields_ = [("n", C.c_int64), ("off", C.POINTER(C.c_int64)), ("idx", C.POINTER(C.c_int32))]


class Csr:
    def __init__(self, ptr):
        self._p = ptr
        c = ptr.contents
        n = int(c.n)
        self.off = np.ctypeslib.as_array(c.off, shape=(n + 1,)).copy()
        tot = int(self.off[-1])
        self.idx = np.ctypeslib.as_array(c.idx, shape=(max(tot, 1),))[:tot].copy()

    def __del__(self):
        try:
            if self._p:
                lib().gxo_csr_free(self._p)
        except Exception:
            pass

    @property
    def ptr(self):
        return self._p


def _mac_setup():
    L = lib()
    if getattr(L, "_mac_ready", False):
        return L
    CP = C.POINTER(_Csr)
    L.gxo_node_radii.argtypes = [_D, _D, _TP, _D]
    L.gxo_mac_lists_build.argtypes = [_TP, _D, C.c_double, C.POINTER(CP), C.POINTER(CP)]
    L.gxo_csr_free.argtypes = [CP]
    L.gxo_compute_fmm_force_mac.argtypes = [_D] * 5 + [_TP, CP, CP, C.c_int64, C.c_double]
    L.gxo_near_split.argtypes = [_TP, _D, C.c_double, CP, C.POINTER(CP), C.POINTER(CP), C.POINTER(CP)]
    L.gxo_compute_fmm_force_wx.argtypes = [_D] * 5 + [_TP, CP, CP, CP, CP, C.c_int64, C.c_double]
    L.gxo_compute_fmm_force_wxb.argtypes = [_D] * 5 + [_TP, CP, CP, CP, CP, C.c_int64, C.c_double, _D, C.c_double]
    L.gxo_body_p2l.argtypes = [_D, _D, _TP, _D, C.c_int64, C.c_int64, C.c_int64, C.c_double]
    L.gxo_body_p2l.restype = C.c_int
    L._mac_ready = True
    return L


def node_radii(b: Bodies, t: Tree) -> np.ndarray:
    r = np.zeros(t.n_nodes)
    _mac_setup().gxo_node_radii(_d(b.x), _d(b.y), t.ptr, _d(r))
    return r


def mac_lists_build(t: Tree, radius: np.ndarray, theta: float):
    L = _mac_setup()
    CP = C.POINTER(_Csr)
    f, n = CP(), CP()
    r = _arr(radius)
    L.gxo_mac_lists_build(t.ptr, _d(r), float(theta), C.byref(f), C.byref(n))
    return Csr(f), Csr(n)


def compute_fmm_force_mac(b: Bodies, t: Tree, far: Csr, near: Csr, p: int, eps: float) -> None:
    _mac_setup().gxo_compute_fmm_force_mac(_d(b.x), _d(b.y), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, far.ptr, near.ptr,
                                           int(p), float(eps))


def near_split(t: Tree, radius: np.ndarray, theta_w: float, near: Csr):
    """The near lists split into (p2p, m2p, p2l) by the leaf-level tests of theta_w."""
    L = _mac_setup()
    CP = C.POINTER(_Csr)
    a, b, c = CP(), CP(), CP()
    r = _arr(radius)
    L.gxo_near_split(t.ptr, _d(r), float(theta_w), near.ptr, C.byref(a), C.byref(b), C.byref(c))
    return Csr(a), Csr(b), Csr(c)


def compute_fmm_force_wx(b: Bodies, t: Tree, far: Csr, near: Csr, m2p: Csr, p2l: Csr, p: int, eps: float) -> None:
    _mac_setup().gxo_compute_fmm_force_wx(_d(b.x), _d(b.y), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, far.ptr,
                                          near.ptr, m2p.ptr if m2p is not None else None,
                                          p2l.ptr if p2l is not None else None, int(p), float(eps))


def body_p2l(b: Bodies, t: Tree, radius: np.ndarray, a: int, s: int, j: int, theta_b: float) -> bool:
    """The per-body test of the body-level P2L: body j of source leaf s joins target leaf
    a's local expansion."""
    r = _arr(radius)
    return bool(_mac_setup().gxo_body_p2l(_d(b.x), _d(b.y), t.ptr, _d(r), int(a), int(s), int(j), float(theta_b)))


def compute_fmm_force_wxb(b: Bodies, t: Tree, far: Csr, near: Csr, m2p: Csr, p2l: Csr, p: int, eps: float,
                          radius: np.ndarray, theta_b: float) -> None:
    """compute_fmm_force_wx with the body-level P2L of the P2P pairs (theta_b > 0)."""
    r = _arr(radius)
    _mac_setup().gxo_compute_fmm_force_wxb(_d(b.x), _d(b.y), _d(b.mass), _d(b.ax), _d(b.ay), t.ptr, far.ptr,
                                           near.ptr, m2p.ptr if m2p is not None else None,
                                           p2l.ptr if p2l is not None else None, int(p), float(eps), _d(r),
                                           float(theta_b))


# ------------------------------------------------------------ N^2 adjoint
def _adj_setup():
    L = lib()
    if getattr(L, "_adj_ready", False):
        return L
    L.gxo_n2_vjp.argtypes = [_D, _D, _D, C.c_int64, C.c_double, _D, _D, _D, _D, _D]
    L.gxo_n2_rollout_grad.argtypes = [_D] * 5 + [C.c_int64, C.c_double, C.c_double, C.c_int64] + [_D] * 9
    L._adj_ready = True
    return L


def n2_vjp(x, y, m, eps, lx, ly):
    x, y, m, lx, ly = (_arr(a) for a in (x, y, m, lx, ly))
    n = x.size
    gx, gy, gm = np.zeros(n), np.zeros(n), np.zeros(n)
    _adj_setup().gxo_n2_vjp(_d(x), _d(y), _d(m), n, float(eps), _d(lx), _d(ly), _d(gx), _d(gy), _d(gm))
    return gx, gy, gm


def n2_rollout_grad(x0, y0, vx0, vy0, m, eps, dt, n_steps, lx, ly, lvx, lvy):
    a = [_arr(v) for v in (x0, y0, vx0, vy0, m)]
    t = [_arr(v) for v in (lx, ly, lvx, lvy)]
    n = a[0].size
    out = [np.zeros(n) for _ in range(5)]
    _adj_setup().gxo_n2_rollout_grad(*[_d(v) for v in a], n, float(eps), float(dt), int(n_steps),
                                     *[_d(v) for v in t], *[_d(o) for o in out])
    return out
