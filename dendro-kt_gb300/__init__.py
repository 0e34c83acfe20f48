"""Python front end of the GB300 k-tree matvec library (ctypes over the C ABI).

The product is the native library built from csrc/ (include/dkt_gb300.h is
its contract); this module only loads it and wraps the calls for tests, the
benchmark and Python users.  Device arrays are torch CUDA tensors, passed by
address.  There is no CPU fallback: without the library or a GPU the calls
raise.
"""
import ctypes
import os

import numpy as np

_PKG = os.path.dirname(os.path.abspath(__file__))
_lib = None

OK, E_ARG, E_CUDA, E_NOMEM, E_UNSUP, E_NOCONV, E_INTERNAL = 0, -1, -2, -3, -4, -5, -6
CURVE_MORTON, CURVE_HILBERT = 0, 1
OP_IDENTITY, OP_HEAT, OP_LAPMASS, OP_CUSTOM, OP_LAPLACE, OP_MASS, OP_HEATVEC = 0, 1, 2, 3, 4, 5, 6
ARITH_AUTO, ARITH_FP64, ARITH_FIXED = 0, 1, 2
TRAVERSAL_REFERENCE, TRAVERSAL_CONFORMING = 0, 1
PREC_FP64, PREC_MIXED = 0, 1
CG_JACOBI, CG_REFERENCE = 1, 2


class DktError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("dkt error %d: %s" % (code, msg))
        self.code = code


def lib_path():
    from . import build as _b  # noqa: F401  (package-relative when imported as a package)
    return _b.LIB


def load(build_if_missing=True):
    """Load libdkt_gb300.so (building it in-tree first if it is missing)."""
    global _lib
    if _lib is not None:
        return _lib
    import importlib.util
    spec = importlib.util.spec_from_file_location("_dkt_build", os.path.join(_PKG, "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    if build_if_missing and not b.up_to_date():
        b.build()
    if not os.path.exists(b.LIB):
        raise RuntimeError("native library missing: %s (run __graft_entry__.build())" % b.LIB)
    L = ctypes.CDLL(b.LIB)
    P, I64, I = ctypes.c_void_p, ctypes.c_int64, ctypes.c_int
    sig = {
        "dkt_last_error": ([], ctypes.c_char_p),
        "dkt_da_create": ([I, I, I, I, P, P, I64, I, P], I),
        "dkt_da_local_nodal_size": ([P], I64),
        "dkt_da_num_elements": ([P], I64),
        "dkt_da_boundary_size": ([P], I64),
        "dkt_da_get_nodes": ([P, P, P], I),
        "dkt_da_get_boundary_ids": ([P, P], I),
        "dkt_da_get_tree": ([P, P, P], I),
        "dkt_da_destroy": ([P], None),
        "dkt_plan_create": ([P, I, P, P], I),
        "dkt_plan_create_ex": ([P, I, P, I, P], I),
        "dkt_plan_create_from_nodes": ([I, I, I, I, P, P, I64, I, P, P], I),
        "dkt_plan_num_nodes": ([P], I64),
        "dkt_plan_stats": ([P, P], I),
        "dkt_plan_export": ([P, P, P, P, P, P], I),
        "dkt_matvec": ([P, P, P, ctypes.c_double, P], I),
        "dkt_fematrix_matvec": ([P, P, P, ctypes.c_double, P], I),
        "dkt_fematrix_matvec_host": ([P, P, P, ctypes.c_double], I),
        "dkt_fematrix_matvec_host_many": ([P, P, P, I, ctypes.c_double], I),
        "dkt_fematrix_matvec_noalloc": ([P, P, P, ctypes.c_double, P], I),
        "dkt_fevector_compute_vec": ([P, P, P, ctypes.c_double, P], I),
        "dkt_diagonal": ([P, P, P], I),
        "dkt_cg_solve": ([P, P, P, I, ctypes.c_double, I, P, P, P], I),
        "dkt_pcg_solve": ([P, P, P, I, I, ctypes.c_double, I, P, P, P, P], I),
        "dkt_matvec_f32": ([P, P, P, P], I),
        "dkt_plan_kernel_timing": ([P, I, P, P], I),
        "dkt_plan_launch_count": ([P, P], I),
        "dkt_plan_set_tile": ([P, I], I),
        "dkt_batch_create": ([P, I, P], I),
        "dkt_plan_num_meshes": ([P, P], I),
        "dkt_plan_mesh_offsets": ([P, P], I),
        "dkt_plan_autotune": ([P, P, P], I),
        "dkt_plan_autotune_ex": ([P, I, P, P, P, P], I),
        "dkt_plan_create_part": ([P, I64, I64, P, I64, P], I),
        "dkt_plan_stats_ex": ([P, P, I], I),
        "dkt_plan_set_arithmetic": ([P, I], I),
        "dkt_plan_destroy": ([P], None),
        "dkt_mesh_gaussian_points": ([I64, I, I, ctypes.c_double, ctypes.c_double, ctypes.c_uint64, P], I),
        "dkt_mesh_tree_from_points": ([P, I64, I, I, I64, P, P, P], I),
        "dkt_mesh_tree_from_points_device": ([P, I64, I, I, I64, P, P, P], I),
        "dkt_mesh_function2octree": ([P, P, I, I, I, I, ctypes.c_double, I, P, P, P], I),
        "dkt_da_set_vector_by_function": ([P, P, P, I, P], I),
        "dkt_write_vtu": ([ctypes.c_char_p, I, I, P, P, I64, P, ctypes.c_char_p], I),
        "dkt_mesh_moving_ball": ([I, I, ctypes.c_double, ctypes.c_double, P, P, P, P, P], I),
        "dkt_free": ([P], None),
        "dkt_mesh_moving_ball_device": ([I, I, ctypes.c_double, ctypes.c_double, P, P, P, P, P], I),
        "dkt_mesh_sphere_shell_device": ([I, I, I, ctypes.c_double, ctypes.c_double, P, P, P, P], I),
        "dkt_mesh_sphere_shell": ([I, I, I, ctypes.c_double, ctypes.c_double, P, P, P, P], I),
        "dkt_curve_tables": ([I, I, P, P, P], I),
        "dkt_server_create": ([I, ctypes.c_double, I, ctypes.c_double, P], I),
        "dkt_server_submit": ([P, I, I, P, P, I64, ctypes.c_uint64, P], I),
        "dkt_server_wait": ([P, I64, P], I),
        "dkt_server_solution": ([P, I64, P, I64], I),
        "dkt_server_release": ([P, I64], I),
        "dkt_server_error": ([P, I64, P, I], I),
        "dkt_server_destroy": ([P], None),
        "dkt_probe_device": ([P], I),
    }
    for name, (args, res) in sig.items():
        f = getattr(L, name)
        f.argtypes = args
        f.restype = res
    _lib = L
    return L


def _p(a):
    return ctypes.c_void_p(a.ctypes.data) if isinstance(a, np.ndarray) else ctypes.c_void_p(int(a.data_ptr()))


def _check(rc):
    if rc != OK:
        raise DktError(rc, load().dkt_last_error().decode())


def _stream(stream):
    if stream is None:
        return None
    return ctypes.c_void_p(int(getattr(stream, "cuda_stream", stream)))


class DA:
    """ot::DA<dim> on one GB300: tree in SFC order, node list, boundary ids."""

    def __init__(self, tree_coords, tree_levels, dim, order=1, max_depth=10, curve=CURVE_MORTON, sorted_tree=False):
        L = load()
        c = np.ascontiguousarray(tree_coords, dtype=np.uint32).reshape(-1, dim)
        lv = np.ascontiguousarray(tree_levels, dtype=np.uint8)
        h = ctypes.c_void_p()
        _check(L.dkt_da_create(dim, order, curve, max_depth, _p(c), _p(lv), lv.size, int(bool(sorted_tree)),
                               ctypes.byref(h)))
        self._h, self.dim, self.order, self.max_depth = h, dim, order, max_depth

    @property
    def handle(self):
        return self._h

    @property
    def n(self):
        return int(load().dkt_da_local_nodal_size(self._h))

    @property
    def n_elem(self):
        return int(load().dkt_da_num_elements(self._h))

    def nodes(self):
        c = np.empty((self.n, self.dim), np.uint32)
        lv = np.empty(self.n, np.uint8)
        _check(load().dkt_da_get_nodes(self._h, _p(c), _p(lv)))
        return c, lv

    def boundary_ids(self):
        nb = int(load().dkt_da_boundary_size(self._h))
        ids = np.empty(max(nb, 1), np.uint32)
        _check(load().dkt_da_get_boundary_ids(self._h, _p(ids)))
        return ids[:nb]

    def tree(self):
        ne = self.n_elem
        c = np.empty((ne, self.dim), np.uint32)
        lv = np.empty(ne, np.uint8)
        _check(load().dkt_da_get_tree(self._h, _p(c), _p(lv)))
        return c, lv

    def set_vector_by_function(self, func, dof=1):
        """DA::setVectorByFunction: func(x) with x [n, min(dim, 3)] node
        coordinates in [0, 1] returns [n, dof]; the nodal vector [n, dof]."""
        out = np.empty((self.n, dof), np.float64)
        err = []

        def cb(xp, n, d, outp, nv, _user):
            try:
                x = np.ctypeslib.as_array(xp, shape=(n, d))
                o = np.ctypeslib.as_array(outp, shape=(n, nv))
                o[...] = np.asarray(func(x), dtype=np.float64).reshape(n, nv)
                return 0
            except Exception as e:   # reported after the call
                err.append(e)
                return 1

        fn = _FIELD_FN(cb)
        rc = load().dkt_da_set_vector_by_function(self._h, ctypes.cast(fn, ctypes.c_void_p), None, int(dof), _p(out))
        if err:
            raise err[0]
        _check(rc)
        return out if dof > 1 else out[:, 0]

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                load().dkt_da_destroy(self._h)
                self._h = None
        except Exception:
            pass


class Matrix:
    """feMatrix<LeafT,dim> over a DA (or a bare node list) with a device plan."""

    def __init__(self, da=None, op=OP_LAPMASS, tables=None, nodes=None, dim=None, order=1, max_depth=10,
                 curve=CURVE_MORTON, traversal=TRAVERSAL_REFERENCE):
        L = load()
        h = ctypes.c_void_p()
        t = None if tables is None else np.ascontiguousarray(tables, dtype=np.float64)
        tp = None if t is None else _p(t)
        if da is not None:
            _check(L.dkt_plan_create_ex(da.handle, op, tp, traversal, ctypes.byref(h)))
        else:
            c = np.ascontiguousarray(nodes[0], dtype=np.uint32).reshape(-1, dim)
            lv = np.ascontiguousarray(nodes[1], dtype=np.uint8)
            _check(L.dkt_plan_create_from_nodes(dim, order, curve, max_depth, _p(c), _p(lv), lv.size, op, tp,
                                                ctypes.byref(h)))
        self._h = h
        self.n = int(L.dkt_plan_num_nodes(h))
        self.dim = da.dim if da is not None else dim
        self.order = da.order if da is not None else order
        self.npe = (self.order + 1) ** self.dim

    @classmethod
    def batch(cls, mats):
        """One block-diagonal plan over several matrices (same dim, order,
        max_depth, operator, traversal, tile size); vectors are concatenated."""
        L = load()
        arr = (ctypes.c_void_p * len(mats))(*[m._h.value for m in mats])
        h = ctypes.c_void_p()
        _check(L.dkt_batch_create(arr, len(mats), ctypes.byref(h)))
        self = cls.__new__(cls)
        self._h = h
        self.n = int(L.dkt_plan_num_nodes(h))
        self.dim, self.order, self.npe = mats[0].dim, mats[0].order, mats[0].npe
        return self

    def stats(self):
        s = np.zeros(9, np.int64)
        _check(load().dkt_plan_stats_ex(self._h, _p(s), 9))
        return dict(zip(["leaves", "hanging_leaves", "stale_slots", "boundary_nodes", "stale_entries",
                         "stale_runs", "stale_longest_run", "stale_longest_run_entries", "fp64_finishes"],
                        s.tolist()))

    def export(self):
        """The flattened traversal as numpy arrays (e2n, info, hidx, p2n, fill)."""
        st = self.stats()
        nl, nh = st["leaves"], st["hanging_leaves"]
        npe = self.npe
        e2n = np.empty((nl, npe), np.int32)
        info = np.empty(nl, np.uint32)
        hidx = np.empty(nl, np.int32)
        p2n = np.empty((max(nh, 1), npe), np.int32)
        fill = np.empty((max(nh, 1), 3), np.uint32)
        _check(load().dkt_plan_export(self._h, _p(e2n), _p(info), _p(hidx), _p(p2n), _p(fill)))
        return e2n, info, hidx, p2n[:nh], fill[:nh]

    def matvec_raw(self, x_dev, y_dev, scale=1.0, stream=None):
        """fem::matvec on device tensors (no boundary handling)."""
        _check(load().dkt_matvec(self._h, _p(x_dev), _p(y_dev), scale, _stream(stream)))

    def matvec(self, x_dev, y_dev, scale=1.0, stream=None):
        """feMatrix::matVec on device tensors."""
        _check(load().dkt_fematrix_matvec(self._h, _p(x_dev), _p(y_dev), scale, _stream(stream)))

    def compute_vec(self, in_dev, out_dev, scale=1.0, stream=None):
        """feVector::computeVec on device tensors (operators OP_HEATVEC, OP_MASS, OP_CUSTOM)."""
        _check(load().dkt_fevector_compute_vec(self._h, _p(in_dev), _p(out_dev), scale, _stream(stream)))

    def matvec_noalloc(self, x_dev, y_dev, scale=1.0, stream=None):
        """feMatrix::matVec that allocates no device memory (fixed 8 MiB scratch per device)."""
        _check(load().dkt_fematrix_matvec_noalloc(self._h, _p(x_dev), _p(y_dev), scale, _stream(stream)))

    def matvec_host(self, x, scale=1.0, out=None):
        """feMatrix::matVec on host arrays (copies in and out; pass pinned
        arrays, e.g. from torch's pin_memory, for direct DMA)."""
        x = np.ascontiguousarray(x, dtype=np.float64)
        y = np.empty(self.n) if out is None else out
        if y.dtype != np.float64 or not y.flags["C_CONTIGUOUS"] or y.size != self.n:
            raise ValueError("out must be a contiguous float64 array of the plan's size")
        _check(load().dkt_fematrix_matvec_host(self._h, _p(x), _p(y), scale))
        return y

    def matvec_host_many(self, xs, ys, scale=1.0):
        """feMatrix::matVec of several host vectors, pipelined: copies of the
        neighbouring products overlap each product (pass pinned arrays)."""
        if len(xs) != len(ys):
            raise ValueError("one output per input")
        for a in list(xs) + list(ys):
            if a.dtype != np.float64 or not a.flags["C_CONTIGUOUS"] or a.size != self.n:
                raise ValueError("vectors must be contiguous float64 arrays of the plan's size")
        k = len(xs)
        xp = (ctypes.c_void_p * max(k, 1))(*[a.ctypes.data for a in xs])
        yp = (ctypes.c_void_p * max(k, 1))(*[a.ctypes.data for a in ys])
        _check(load().dkt_fematrix_matvec_host_many(self._h, xp, yp, k, scale))
        return ys

    def set_arithmetic(self, mode):
        """ARITH_AUTO (fixed point where it applies), ARITH_FP64 or ARITH_FIXED."""
        _check(load().dkt_plan_set_arithmetic(self._h, mode))

    def set_tile(self, tile_leaves):
        """Leaves per tile of the Q1 kernels (0: untiled kernel)."""
        _check(load().dkt_plan_set_tile(self._h, int(tile_leaves)))

    def launch_count(self):
        """Kernels launched so far by this matrix's products and solves."""
        n = ctypes.c_int64()
        _check(load().dkt_plan_launch_count(self._h, ctypes.byref(n)))
        return n.value

    def kernel_timing(self, enable):
        """Close the current timing window; returns (total kernel ms, launches)."""
        ms = ctypes.c_double(0.0)
        n = ctypes.c_int64(0)
        _check(load().dkt_plan_kernel_timing(self._h, int(bool(enable)), ctypes.byref(ms), ctypes.byref(n)))
        return ms.value, n.value

    def diagonal(self, d_dev, stream=None):
        _check(load().dkt_diagonal(self._h, _p(d_dev), _stream(stream)))

    def cg(self, b_dev, x_dev, max_iter=10000, tol=1e-10, jacobi=True, reference=False, stream=None):
        """CG on device tensors.  reference=True: HeatMat::cgSolve itself (no
        preconditioner, relative L-infinity stop).  Returns (iterations,
        final relative residual, converged)."""
        it = ctypes.c_int(0)
        rr = ctypes.c_double(0.0)
        flags = CG_REFERENCE if reference else (CG_JACOBI if jacobi else 0)
        rc = load().dkt_cg_solve(self._h, _p(b_dev), _p(x_dev), max_iter, tol, flags,
                                 ctypes.byref(it), ctypes.byref(rr), _stream(stream))
        if rc not in (OK, E_NOCONV):
            _check(rc)
        return it.value, rr.value, rc == OK

    def pcg(self, b_dev, x_dev, precision=0, max_iter=100000, tol=1e-10, jacobi=True, stream=None):
        """Device-resident Jacobi-PCG (precision PREC_FP64) or mixed-precision
        refinement (PREC_MIXED).  Returns (iterations, refinements, relres,
        converged); for a batch the first three are per-mesh arrays."""
        m = self.num_meshes()
        it, ref, rr = np.zeros(m, np.int32), np.zeros(m, np.int32), np.zeros(m)
        rc = load().dkt_pcg_solve(self._h, _p(b_dev), _p(x_dev), int(precision), int(max_iter), float(tol),
                                  int(bool(jacobi)), _p(it), _p(ref), _p(rr), _stream(stream))
        if rc not in (OK, E_NOCONV):
            _check(rc)
        if m == 1:
            return int(it[0]), int(ref[0]), float(rr[0]), rc == OK
        return it, ref, rr, rc == OK

    def num_meshes(self):
        n = ctypes.c_int(0)
        _check(load().dkt_plan_num_meshes(self._h, ctypes.byref(n)))
        return n.value

    def mesh_offsets(self):
        m = self.num_meshes()
        o = np.zeros(m + 1, np.int64)
        _check(load().dkt_plan_mesh_offsets(self._h, _p(o)))
        return o

    def autotune(self, arith=0):
        """Keeps the fastest launch shape for the FP64 (arith 0) or binary32
        (arith 1) product; returns (tile, persistent, ms per product, times of
        all candidates: untiled, then per tile size plain and persistent)."""
        t, p, ms = ctypes.c_int(0), ctypes.c_int(0), ctypes.c_double(0.0)
        times = np.zeros(7)
        _check(load().dkt_plan_autotune_ex(self._h, int(arith), ctypes.byref(t), ctypes.byref(p), ctypes.byref(ms),
                                           _p(times)))
        return t.value, bool(p.value), ms.value, times

    def matvec_f32(self, x_dev, y_dev, stream=None):
        """Binary32 feMatrix product (Q1 built-in operators)."""
        _check(load().dkt_matvec_f32(self._h, _p(x_dev), _p(y_dev), _stream(stream)))

    def __del__(self):
        try:
            if getattr(self, "_h", None):
                load().dkt_plan_destroy(self._h)
                self._h = None
        except Exception:
            pass


def probe_device():
    """FP64 FMA / FP64 add / FP32 FMA / int64 add throughput of the current GPU."""
    out = np.zeros(4)
    _check(load().dkt_probe_device(_p(out)))
    return dict(zip(["fp64_fma_tflops", "fp64_add_tops", "fp32_fma_tflops", "int64_add_tops"], out.tolist()))


def gaussian_points(n, dim, max_depth, mean=0.5, sd=0.1, seed=0):
    out = np.empty((n, dim), np.uint32)
    _check(load().dkt_mesh_gaussian_points(n, dim, max_depth, mean, sd, seed, _p(out)))
    return out


def _take_cells(n, c, lv, dim):
    L = load()
    try:
        coords = np.ctypeslib.as_array(ctypes.cast(c, ctypes.POINTER(ctypes.c_uint32)), shape=(n.value * dim,)).copy()
        levels = np.ctypeslib.as_array(ctypes.cast(lv, ctypes.POINTER(ctypes.c_uint8)), shape=(n.value,)).copy()
    finally:
        L.dkt_free(c)
        L.dkt_free(lv)
    return coords.reshape(-1, dim), levels


def tree_from_points(points, dim, max_depth, max_pts=1, device=False):
    """Complete tree with at most max_pts points per leaf, 2:1 balanced
    (device=True builds it on the GPU, False on the host; the trees are equal)."""
    pts = np.ascontiguousarray(points, dtype=np.uint32).reshape(-1, dim)
    n, c, lv = ctypes.c_int64(0), ctypes.c_void_p(), ctypes.c_void_p()
    fn = load().dkt_mesh_tree_from_points_device if device else load().dkt_mesh_tree_from_points
    _check(fn(_p(pts), pts.shape[0], dim, max_depth, max_pts, ctypes.byref(n), ctypes.byref(c), ctypes.byref(lv)))
    return _take_cells(n, c, lv, dim)


_FIELD_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.POINTER(ctypes.c_double), ctypes.c_int64, ctypes.c_int,
                             ctypes.POINTER(ctypes.c_double), ctypes.c_int, ctypes.c_void_p)


def function2octree(func, n_vars, dim, max_depth, order=1, interp_tol=1e-3, balance=True):
    """ot::function2Octree (balance=False) or the tree of ot::DA(func, ...)
    (balance=True), built on the GPU.  func(x) takes points x [n, dim] in
    [0, 1]^dim and returns the fields' values [n, n_vars]; it is called on
    batches of points."""
    err = []

    def cb(xp, n, d, outp, nv, _user):
        try:
            x = np.ctypeslib.as_array(xp, shape=(n, d))
            out = np.ctypeslib.as_array(outp, shape=(n, nv))
            out[...] = np.asarray(func(x), dtype=np.float64).reshape(n, nv)
            return 0
        except Exception as e:   # reported after the call
            err.append(e)
            return 1

    fn = _FIELD_FN(cb)
    n, c, lv = ctypes.c_int64(0), ctypes.c_void_p(), ctypes.c_void_p()
    rc = load().dkt_mesh_function2octree(ctypes.cast(fn, ctypes.c_void_p), None, int(n_vars), int(dim),
                                         int(max_depth), int(order), float(interp_tol), 1 if balance else 0,
                                         ctypes.byref(n), ctypes.byref(c), ctypes.byref(lv))
    if err:
        raise err[0]
    _check(rc)
    return _take_cells(n, c, lv, dim)


def write_vtu(path, coords, levels, dim, max_depth, cell_values=None, name="value"):
    """io::vtk::oct2vtu: write the tree (dim 2 or 3) as a VTU file."""
    c = np.ascontiguousarray(coords, dtype=np.uint32).reshape(-1, dim)
    lv = np.ascontiguousarray(levels, dtype=np.uint8)
    cv = None if cell_values is None else np.ascontiguousarray(cell_values, dtype=np.float64)
    if cv is not None and cv.size != lv.size:
        raise ValueError("one cell value per cell")
    _check(load().dkt_write_vtu(os.fsencode(path), int(dim), int(max_depth), _p(c), _p(lv), lv.size,
                                None if cv is None else _p(cv), name.encode()))


def curve_tables(curve, dim):
    """(rot, ht) rotation tables of CURVE_MORTON or CURVE_HILBERT for dim 2..4."""
    rot = np.zeros(192 * 32, np.int8)
    ht = np.zeros(192 * 16, np.int32)
    n = ctypes.c_int(0)
    _check(load().dkt_curve_tables(int(curve), int(dim), _p(rot), _p(ht), ctypes.byref(n)))
    nc = 1 << dim
    return rot[:n.value * 2 * nc].copy(), ht[:n.value * nc].copy()


def sphere_shell_tree(dim, max_depth, level, centre, radius, halfwidth=None, device=True):
    """2:1-balanced tree refined to `level` on a sphere shell (device=True
    builds it on the GPU, False on the host; the trees are equal)."""
    if halfwidth is None:
        halfwidth = 2.0 ** -level
    c = np.ascontiguousarray(centre, dtype=np.float64)
    n, cp, lv = ctypes.c_int64(0), ctypes.c_void_p(), ctypes.c_void_p()
    fn = load().dkt_mesh_sphere_shell_device if device else load().dkt_mesh_sphere_shell
    _check(fn(dim, max_depth, level, float(radius), float(halfwidth), _p(c),
                                               ctypes.byref(n), ctypes.byref(cp), ctypes.byref(lv)))
    return _take_cells(n, cp, lv, dim)


def moving_ball_tree(max_depth, level, radius=0.2, halfwidth=None, c0=(0.3, 0.3, 0.3), c1=(0.7, 0.7, 0.7),
                     device=False):
    """Spacetime moving-ball tree (dim 4); device=True builds it on the GPU."""
    if halfwidth is None:
        halfwidth = 2.0 ** -level
    a0 = np.ascontiguousarray(c0, dtype=np.float64)
    a1 = np.ascontiguousarray(c1, dtype=np.float64)
    n, c, lv = ctypes.c_int64(0), ctypes.c_void_p(), ctypes.c_void_p()
    fn = load().dkt_mesh_moving_ball_device if device else load().dkt_mesh_moving_ball
    _check(fn(max_depth, level, radius, halfwidth, _p(a0), _p(a1), ctypes.byref(n), ctypes.byref(c),
              ctypes.byref(lv)))
    return _take_cells(n, c, lv, 4)


class _SolveReport(ctypes.Structure):
    _fields_ = [("rc", ctypes.c_int), ("dim", ctypes.c_int), ("n_elem", ctypes.c_int64), ("n_nodes", ctypes.c_int64),
                ("iterations", ctypes.c_int), ("refinements", ctypes.c_int), ("relres", ctypes.c_double),
                ("t_submit", ctypes.c_double), ("t_admit", ctypes.c_double), ("t_start", ctypes.c_double),
                ("t_done", ctypes.c_double), ("device_bytes", ctypes.c_int64), ("est_bytes", ctypes.c_double)]


class Server:
    """Request loop for Q1 Poisson solves (native worker threads, admission
    against a device-memory budget, concurrent requests on separate streams)."""

    def __init__(self, workers=4, budget_bytes=150e9, precision=PREC_MIXED, tol=1e-10):
        h = ctypes.c_void_p()
        _check(load().dkt_server_create(int(workers), float(budget_bytes), int(precision), float(tol),
                                        ctypes.byref(h)))
        self._h = h

    def submit(self, tree_coords, tree_levels, dim, max_depth, seed=0):
        c = np.ascontiguousarray(tree_coords, dtype=np.uint32).reshape(-1, dim)
        lv = np.ascontiguousarray(tree_levels, dtype=np.uint8)
        t = ctypes.c_int64(0)
        _check(load().dkt_server_submit(self._h, dim, max_depth, _p(c), _p(lv), lv.size, ctypes.c_uint64(seed),
                                         ctypes.byref(t)))
        return t.value

    def wait(self, ticket, solution=True):
        rep = _SolveReport()
        _check(load().dkt_server_wait(self._h, ctypes.c_int64(ticket), ctypes.byref(rep)))
        out = {k: getattr(rep, k) for k, _ in _SolveReport._fields_}
        if rep.rc not in (OK, E_NOCONV):
            buf = ctypes.create_string_buffer(512)
            load().dkt_server_error(self._h, ctypes.c_int64(ticket), buf, 512)
            out["error"] = buf.value.decode(errors="replace")
        if solution and rep.n_nodes > 0:
            x = np.empty(rep.n_nodes)
            _check(load().dkt_server_solution(self._h, ctypes.c_int64(ticket), _p(x), ctypes.c_int64(x.size)))
            out["x"] = x
        load().dkt_server_release(self._h, ctypes.c_int64(ticket))
        return out

    def close(self):
        if getattr(self, "_h", None):
            load().dkt_server_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def cluster_points(n, dim, max_depth, seed, sd=0.05):
    """n points around 1-4 Gaussian clusters (centres uniform in
    [0.2, 0.8]^dim, standard deviation sd, numpy PCG64 stream of `seed`),
    clipped to the unit cube, as integer coordinates at max_depth."""
    rng = np.random.default_rng(seed)
    k = int(rng.integers(1, 5))
    centres = rng.uniform(0.2, 0.8, size=(k, dim))
    which = rng.integers(0, k, size=n)
    p = np.clip(centres[which] + rng.normal(0.0, sd, size=(n, dim)), 0.0, 1.0 - 2.0 ** -max_depth)
    return np.floor(p * (1 << max_depth)).astype(np.uint32)


def sine_load(da, noise_sd=0.1, seed=3):
    """Nodal load f = prod_d sin(pi x_d) + N(0, noise_sd^2) noise (numpy
    PCG64 stream of `seed`) at the DA's nodes, in DA node order."""
    c, _ = da.nodes()
    x = c.astype(np.float64) * (0.5 ** da.max_depth)
    f = np.prod(np.sin(np.pi * x), axis=1)
    if noise_sd:
        f = f + np.random.default_rng(seed).normal(0.0, noise_sd, size=len(f))
    return f


def uniform_pm1(seed, n):
    """Nodal vector x_i = 2u - 1 from the counter-based stream used everywhere
    in this project (top 53 bits of splitmix64(seed * K + i))."""
    def splitmix64(z):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))
    with np.errstate(over="ignore"):
        r = splitmix64(np.uint64(seed) * np.uint64(0xD1B54A32D192ED03) + np.arange(n, dtype=np.uint64))
    return 2.0 * ((r >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)) - 1.0


def uniform_pm1_coords(seed, coords):
    """Nodal vector keyed by node coordinates instead of DA position: the same
    node gets the same value in any node order (Morton or Hilbert DA, any
    partition).  x = 2u - 1, u from splitmix64 chained over the coordinates."""
    def splitmix64(z):
        z = z + np.uint64(0x9E3779B97F4A7C15)
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))
    c = np.asarray(coords, dtype=np.uint64)
    with np.errstate(over="ignore"):
        h = np.full(c.shape[0], np.uint64(seed) * np.uint64(0xD1B54A32D192ED03), np.uint64)
        for d in range(c.shape[1]):
            h = splitmix64(h ^ c[:, d])
    return 2.0 * ((h >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)) - 1.0


from . import partition  # noqa: E402  (multi-part meshes: partition maps and ghost exchange)
