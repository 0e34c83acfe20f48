"""ctypes front end of the CPU oracle (oracle/port/dkt_oracle.cpp).

TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
CPU-baseline leg may import this module; the product never does.  The library
is a restatement of the reference algorithms (SFC_Tree, SFC_NodeSort,
ot::DA, fem::matvec, HeatMat) and is pinned against the reference build on the
golden fixtures in tests/golden/.
"""
import ctypes
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "_build", "libdkt_oracle.so")
SRC_PATH = os.path.join(_HERE, "port", "dkt_oracle.cpp")

_lib = None


def build(force=False):
    """Compile the oracle library with the host C++ compiler."""
    os.makedirs(os.path.dirname(LIB_PATH), exist_ok=True)
    if (not force and os.path.exists(LIB_PATH)
            and os.path.getmtime(LIB_PATH) >= os.path.getmtime(SRC_PATH)):
        return LIB_PATH
    cmd = ["g++", "-O2", "-std=c++17", "-shared", "-fPIC", SRC_PATH, "-o", LIB_PATH]
    subprocess.run(cmd, check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        P = ctypes.c_void_p
        L.dkto_last_error.restype = ctypes.c_char_p
        L.dkto_set_curve.argtypes = [ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int]
        L.dkto_tree_balance.argtypes = [ctypes.c_int, P, ctypes.c_int64, ctypes.c_int64, P]
        L.dkto_tree_fetch.argtypes = [P, P]
        L.dkto_tree_sort.argtypes = [ctypes.c_int, P, P, ctypes.c_int64]
        L.dkto_da_create.argtypes = [ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P, ctypes.c_int64, P]
        L.dkto_da_num_nodes.argtypes = [P]
        L.dkto_da_num_nodes.restype = ctypes.c_int64
        L.dkto_da_num_bdry.argtypes = [P]
        L.dkto_da_num_bdry.restype = ctypes.c_int64
        L.dkto_da_nodes.argtypes = [P, P, P, P]
        L.dkto_da_refel.argtypes = [P, P, P, P, P, P]
        L.dkto_da_destroy.argtypes = [P]
        L.dkto_da_destroy.restype = None
        L.dkto_matvec_raw.argtypes = [P, P, P]
        L.dkto_fematrix_matvec.argtypes = [P, P, P]
        L.dkto_last_stats.argtypes = [P, P]
        L.dkto_set_stale_mode.argtypes = [ctypes.c_int]
        L.dkto_set_conforming.argtypes = [ctypes.c_int]
        L.dkto_cg.argtypes = [P, P, P, P, ctypes.c_int, ctypes.c_double, P, P]
        L.dkto_cg_ref.argtypes = [P, P, P, ctypes.c_int, ctypes.c_double, P, P, P]
        L.dkto_moving_ball.argtypes = [ctypes.c_int, ctypes.c_double, ctypes.c_double, P, P, ctypes.c_int,
                                        ctypes.c_int64, P]
        _lib = L
    return _lib


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(rc):
    if rc != 0:
        raise RuntimeError("oracle: " + lib().dkto_last_error().decode())


def set_curve(dim, max_depth, rot=None, ht=None):
    """Select Morton (rot is None) or a rotation-table curve for later calls."""
    if rot is None:
        _check(lib().dkto_set_curve(dim, max_depth, None, None, 0))
    else:
        rot = np.ascontiguousarray(rot, dtype=np.int8)
        ht = np.ascontiguousarray(ht, dtype=np.int32)
        nrot = ht.size >> dim
        _check(lib().dkto_set_curve(dim, max_depth, _ptr(rot), _ptr(ht), nrot))


def set_stale_mode(mode):
    """0: parent-buffer slots keep earlier leaves' values (the reference's
    static buffer); 1: unfilled slots read as zero."""
    _check(lib().dkto_set_stale_mode(int(mode)))


def set_conforming(on):
    """0: the reference's traversal; 1: its conforming variant (parent values
    from every node on the parent lattice, unmasked transpose: P^T K P)."""
    _check(lib().dkto_set_conforming(int(on)))


def tree_balance(points, dim, max_pts=1):
    """SFC_Tree::locTreeBalancing over level-max_depth points."""
    pts = np.ascontiguousarray(points, dtype=np.uint32).reshape(-1, dim)
    n = ctypes.c_int64(0)
    _check(lib().dkto_tree_balance(dim, _ptr(pts), pts.shape[0], max_pts, ctypes.byref(n)))
    c = np.empty((n.value, dim), np.uint32)
    lv = np.empty(n.value, np.uint8)
    _check(lib().dkto_tree_fetch(_ptr(c), _ptr(lv)))
    return c, lv


def moving_ball_tree(level, radius=0.2, halfwidth=None, c0=(0.3, 0.3, 0.3), c1=(0.7, 0.7, 0.7), part_level=0,
                     part_index=0):
    """The spacetime moving-ball mesh (dim 4, max_depth of set_curve),
    2:1 balanced; with part_level > 0 only the level-part_level cell of
    Morton index part_index is refined (one partition of the mesh).
    Returns (coords, levels) in no particular order."""
    if halfwidth is None:
        halfwidth = 2.0 ** -level
    a0 = np.ascontiguousarray(c0, dtype=np.float64)
    a1 = np.ascontiguousarray(c1, dtype=np.float64)
    n = ctypes.c_int64(0)
    _check(lib().dkto_moving_ball(level, radius, halfwidth, _ptr(a0), _ptr(a1), part_level, part_index,
                                  ctypes.byref(n)))
    c = np.empty((n.value, 4), np.uint32)
    lv = np.empty(n.value, np.uint8)
    _check(lib().dkto_tree_fetch(_ptr(c), _ptr(lv)))
    return c, lv


def tree_sort(coords, levels, dim):
    c = np.ascontiguousarray(coords, dtype=np.uint32).reshape(-1, dim).copy()
    lv = np.ascontiguousarray(levels, dtype=np.uint8).copy()
    _check(lib().dkto_tree_sort(dim, _ptr(c), _ptr(lv), lv.size))
    return c, lv


class DA:
    """ot::DA + feMatrix restated: node list, boundary ids, matvec."""

    def __init__(self, tree_coords, tree_levels, dim, order, op):
        self.dim, self.order, self.op = dim, order, op
        c = np.ascontiguousarray(tree_coords, dtype=np.uint32).reshape(-1, dim)
        lv = np.ascontiguousarray(tree_levels, dtype=np.uint8)
        h = ctypes.c_void_p()
        _check(lib().dkto_da_create(dim, order, op, _ptr(c), _ptr(lv), lv.size, ctypes.byref(h)))
        self._h = h
        n = lib().dkto_da_num_nodes(h)
        nb = lib().dkto_da_num_bdry(h)
        self.node_coords = np.empty((n, dim), np.uint32)
        self.node_levels = np.empty(n, np.uint8)
        self.bdry = np.empty(nb, np.uint32)
        _check(lib().dkto_da_nodes(h, _ptr(self.node_coords), _ptr(self.node_levels), _ptr(self.bdry)))

    @property
    def n(self):
        return self.node_levels.size

    def refel(self):
        m = self.order + 1
        mats = [np.empty((m, m)) for _ in range(4)] + [np.empty(m)]
        _check(lib().dkto_da_refel(self._h, *[_ptr(a) for a in mats]))
        return dict(zip(["ip0", "ip1", "Q1d", "Dg", "W"], mats))

    def matvec_raw(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        _check(lib().dkto_matvec_raw(self._h, _ptr(x), _ptr(y)))
        return y

    def matvec(self, x):
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n)
        _check(lib().dkto_fematrix_matvec(self._h, _ptr(x), _ptr(y)))
        return y

    def stats(self):
        s = np.zeros(6, np.int64)
        _check(lib().dkto_last_stats(self._h, _ptr(s)))
        return dict(zip(["leaves", "hanging_leaves", "stale_reads", "aliased", "max_level", "ref_errors"], s.tolist()))

    def cg(self, b, x0=None, diag=None, max_iter=10000, tol=1e-10):
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0)
        d = None if diag is None else np.ascontiguousarray(diag, dtype=np.float64)
        _check(lib().dkto_cg(self._h, _ptr(b), _ptr(x), None if d is None else _ptr(d),
                             max_iter, tol, ctypes.byref(it), ctypes.byref(rr)))
        return x, it.value, rr.value

    def cg_ref(self, b, x0=None, max_iter=1000, tol=1e-10):
        """HeatMat::cgSolve: unpreconditioned, relative L-infinity stop.
        Returns (x, iterations, final relative residual, status)."""
        b = np.ascontiguousarray(b, dtype=np.float64)
        x = np.zeros(self.n) if x0 is None else np.array(x0, dtype=np.float64)
        it, st = ctypes.c_int(0), ctypes.c_int(0)
        rr = ctypes.c_double(0)
        _check(lib().dkto_cg_ref(self._h, _ptr(b), _ptr(x), max_iter, tol, ctypes.byref(it), ctypes.byref(rr),
                                 ctypes.byref(st)))
        return x, it.value, rr.value, st.value

    def __del__(self):
        try:
            if self._h:
                lib().dkto_da_destroy(self._h)
        except Exception:
            pass


def splitmix64(z):
    z = (np.asarray(z, dtype=np.uint64) + np.uint64(0x9E3779B97F4A7C15))
    z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
    z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
    return z ^ (z >> np.uint64(31))


def uniform_pm1(seed, n):
    """x_i = 2*u_i - 1 with u_i the top 53 bits of splitmix64(seed*K + i)."""
    with np.errstate(over="ignore"):
        base = np.uint64(seed) * np.uint64(0xD1B54A32D192ED03)
        r = splitmix64(base + np.arange(n, dtype=np.uint64))
    return 2.0 * ((r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)) - 1.0
