"""CPU-side checks of the native library: it loads, exports every function the
C ABI headers declare, rejects bad arguments, and its host-side mesh
generators agree with the oracle's restatement of the reference's tree
construction and 2:1 balancing (SFC_Tree::locTreeBalancing)."""
import ctypes
import os
import re

import numpy as np
import pytest

import __graft_entry__ as ge
import oracle_port as orc

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    names = []
    for h in ("dkt_gb300.h", "dkt_gb300_mesh.h"):
        txt = open(os.path.join(REPO, "include", h)).read()
        txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?[a-z_0-9]+\s*\*?\s*(dkt_[a-z_0-9]+)\s*\(", txt, flags=re.M)
    return sorted(set(names))


@pytest.fixture(scope="module")
def dkt():
    return ge.load_package()


def test_library_exports_all_declared_symbols(dkt):
    L = dkt.load()
    names = _declared()
    assert len(names) >= 20
    for n in names:
        assert hasattr(L, n), n


def test_error_codes_without_device(dkt):
    L = dkt.load()
    h = ctypes.c_void_p()
    c = np.zeros((1, 3), np.uint32)
    lv = np.zeros(1, np.uint8)
    # bad dim, bad order, Hilbert unavailable, misaligned anchor
    assert L.dkt_da_create(5, 1, 0, 10, dkt._p(c), dkt._p(lv), 1, 1, ctypes.byref(h)) == dkt.E_ARG
    assert L.dkt_da_create(3, 3, 0, 10, dkt._p(c), dkt._p(lv), 1, 1, ctypes.byref(h)) == dkt.E_UNSUP
    assert L.dkt_da_create(3, 1, 7, 10, dkt._p(c), dkt._p(lv), 1, 1, ctypes.byref(h)) == dkt.E_ARG   # unknown curve
    c2 = np.array([[3, 0, 0]], np.uint32)
    lv2 = np.array([2], np.uint8)
    assert L.dkt_da_create(3, 1, 0, 10, dkt._p(c2), dkt._p(lv2), 1, 1, ctypes.byref(h)) == dkt.E_ARG
    assert b"aligned" in L.dkt_last_error()
    assert L.dkt_plan_create(None, 2, None, ctypes.byref(h)) == dkt.E_ARG
    # entry points added for feVector, DA(func) and the device tree builder:
    # argument errors come back before any device work
    x = np.zeros(4)
    assert L.dkt_fevector_compute_vec(None, dkt._p(x), dkt._p(x), ctypes.c_double(1.0), None) == dkt.E_ARG
    n = ctypes.c_int64()
    pc, pl = ctypes.c_void_p(), ctypes.c_void_p()
    pts = np.zeros((2, 3), np.uint32)
    assert L.dkt_mesh_tree_from_points_device(dkt._p(pts), 2, 5, 8, 1, ctypes.byref(n), ctypes.byref(pc),
                                              ctypes.byref(pl)) == dkt.E_ARG          # dim 5
    assert L.dkt_mesh_tree_from_points_device(dkt._p(pts), 2, 3, 8, 0, ctypes.byref(n), ctypes.byref(pc),
                                              ctypes.byref(pl)) == dkt.E_ARG          # max_pts 0
    far = np.full((1, 3), 1 << 9, np.uint32)
    assert L.dkt_mesh_tree_from_points_device(dkt._p(far), 1, 3, 8, 1, ctypes.byref(n), ctypes.byref(pc),
                                              ctypes.byref(pl)) == dkt.E_ARG          # outside 2^8
    assert b"outside" in L.dkt_last_error()
    assert L.dkt_mesh_function2octree(None, None, 1, 3, 8, 1, ctypes.c_double(1e-3), 1, ctypes.byref(n),
                                      ctypes.byref(pc), ctypes.byref(pl)) == dkt.E_ARG   # no callback
    cb = dkt._FIELD_FN(lambda *a: 0)
    fp = ctypes.cast(cb, ctypes.c_void_p)
    assert L.dkt_mesh_function2octree(fp, None, 1, 3, 8, 3, ctypes.c_double(1e-3), 1, ctypes.byref(n),
                                      ctypes.byref(pc), ctypes.byref(pl)) == dkt.E_ARG   # order 3
    assert L.dkt_mesh_function2octree(fp, None, 0, 3, 8, 1, ctypes.c_double(1e-3), 1, ctypes.byref(n),
                                      ctypes.byref(pc), ctypes.byref(pl)) == dkt.E_ARG   # no fields


@pytest.mark.parametrize("dim,n,md", [(2, 300, 8), (3, 500, 9), (4, 80, 6)])
def test_tree_builder_matches_reference_balancing(dkt, dim, n, md):
    pts = dkt.gaussian_points(n, dim, md, seed=3)
    tc, tl = dkt.tree_from_points(pts, dim, md)
    orc.set_curve(dim, md)
    sc, sl = orc.tree_sort(tc, tl, dim)
    rc, rl = orc.tree_balance(pts, dim)
    assert np.array_equal(sc, rc) and np.array_equal(sl, rl)


def test_gaussian_points_deterministic(dkt):
    a = dkt.gaussian_points(1000, 3, 10, seed=0)
    b = dkt.gaussian_points(1000, 3, 10, seed=0)
    assert np.array_equal(a, b)
    x = a.astype(np.float64) / 1024.0
    assert abs(x.mean() - 0.5) < 0.02 and abs(x.std() - 0.1) < 0.02


def test_moving_ball_is_complete(dkt):
    tc, tl = dkt.moving_ball_tree(max_depth=6, level=4)
    dim, md = 4, 6
    orc.set_curve(dim, md)
    sc, sl = orc.tree_sort(tc, tl, dim)
    # complete: the cells' volumes sum to the domain's (2:1 balance is checked
    # in test_tree_properties.py)
    vol = np.sum((2.0 ** -sl.astype(np.float64)) ** dim)
    assert abs(vol - 1.0) < 1e-12
    assert sl.max() == 4


def _vtu_arrays(path):
    import base64
    import xml.etree.ElementTree as ET
    types = {"UInt32": np.uint32, "UInt64": np.uint64, "UInt8": np.uint8, "Float64": np.float64}
    out = {}
    for da in ET.parse(path).getroot().iter("DataArray"):
        raw = base64.b64decode(da.text.strip())
        nbytes = int(np.frombuffer(raw[:4], np.uint32)[0])
        assert nbytes == len(raw) - 4
        out[da.get("Name")] = np.frombuffer(raw[4:], types[da.get("type")])
    return out


@pytest.mark.parametrize("dim", [2, 3])
def test_write_vtu_roundtrip(dkt, tmp_path, dim):
    """oct2vtu: every cell's corners, VTK corner order, cell types and cell
    values come back from the file."""
    md = 6
    pts = dkt.gaussian_points(200, dim, md, seed=3)
    c, l = dkt.tree_from_points(pts, dim, md)
    path = str(tmp_path / "tree.vtu")
    dkt.write_vtu(path, c, l, dim, md, cell_values=l.astype(np.float64), name="level")
    a = _vtu_arrays(path)
    nv = 1 << dim
    P = a["Position"].reshape(-1, 3)
    assert P.shape[0] == len(l) * nv
    conn = a["connectivity"].reshape(-1, nv)
    assert np.array_equal(a["offsets"], nv * np.arange(1, len(l) + 1))
    assert np.all(a["types"] == (12 if dim == 3 else 9))
    assert np.array_equal(a["level"], l.astype(np.float64))
    assert np.array_equal(a["cell_level"], l.astype(np.uint32))
    assert np.all(a["mpi_rank"] == 0)
    lens = (1 << (md - l.astype(np.int64)))
    first = P[conn[:, 0]][:, :dim].astype(np.int64)
    assert np.array_equal(first, c.astype(np.int64))
    # counter-clockwise around the bottom face: +x, then +y, then -x
    assert np.array_equal(P[conn[:, 1]][:, 0].astype(np.int64) - first[:, 0], lens)
    assert np.array_equal(P[conn[:, 2]][:, 1].astype(np.int64) - first[:, 1], lens)
    assert np.array_equal(P[conn[:, 3]][:, 0].astype(np.int64), first[:, 0])
    if dim == 3:
        assert np.array_equal(P[conn[:, 4]][:, 2].astype(np.int64) - first[:, 2], lens)
    else:
        assert np.all(P[:, 2] == 0)


@pytest.mark.parametrize("curve", ["morton", "hilbert"])
def test_write_vtu_matches_reference_oct2vtu(dkt, tmp_path, curve):
    """The reference's io::vtk::oct2vtu, run on the same tree in the same
    order (tests/golden/vtu, from its ASCII build): every data array equal."""
    g = np.load(os.path.join(os.path.dirname(__file__), "golden", "vtu", f"{curve}_d3_gauss300.npz"))
    path = str(tmp_path / "tree.vtu")
    dkt.write_vtu(path, g["tree_coords"], g["tree_levels"], 3, int(g["md"]))
    a = _vtu_arrays(path)
    assert sorted(a) == sorted(["Position", "connectivity", "offsets", "types", "mpi_rank", "cell_level"])
    for name in a:
        assert a[name].dtype == g[name].dtype, name
        assert np.array_equal(a[name], g[name]), name


def test_write_vtu_rejects_4d(dkt, tmp_path):
    L = dkt.load()
    c = np.zeros((1, 4), np.uint32)
    l = np.zeros(1, np.uint8)
    rc = L.dkt_write_vtu(str(tmp_path / "x.vtu").encode(), 4, 5, c.ctypes.data, l.ctypes.data, 1, None, b"v")
    assert rc == dkt.E_ARG
