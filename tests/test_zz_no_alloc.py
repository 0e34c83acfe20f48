"""The allocation-free feMatrix::matVec entry point.

dkt_fematrix_matvec_noalloc serves callers that cannot allocate device memory
while a product runs (a loop that reserved its device-memory budget up front,
or code that must not let cudaMalloc/cudaFree stall the device).  Its scratch
lives in a fixed device array; these tests call it through the C ABI and
check it against the regular entry point on two calls in a row, and that it
refuses plans larger than its scratch.  This file is collected last."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
import trees

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def dkt():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return ge.load_package()


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("dim,order,op", [(3, 1, 2), (4, 1, 2), (3, 2, 2), (2, 1, 0)])
def test_noalloc_matches_regular_entry_point_twice(dkt, dim, order, op):
    import torch
    md = 9
    pts = dkt.gaussian_points(1500 if dim < 4 else 200, dim, md - 1, seed=11)
    tc, tl = dkt.tree_from_points(pts, dim, md - 1)
    tc = tc << np.uint32(1)
    da = dkt.DA(tc, tl, dim, order=order, max_depth=md)
    A = dkt.Matrix(da, op=op)
    L = dkt.load()
    for call, seed in enumerate((21, 22)):
        x = torch.from_numpy(dkt.uniform_pm1(seed, da.n)).cuda()
        y_ref = torch.empty_like(x)
        y_new = torch.full_like(x, float("nan"))
        A.matvec(x, y_ref)
        rc = L.dkt_fematrix_matvec_noalloc(A._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_new.data_ptr()),
                                           1.0, None)
        assert rc == dkt.OK, L.dkt_last_error()
        torch.cuda.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert _rel(a, b) <= TOL, (call, _rel(a, b))


def test_noalloc_rejects_plans_beyond_its_scratch(dkt):
    dim, md, L = 3, 8, 7      # 129^3 = 2,146,689 nodes > 1,048,576
    c, lv = trees.example2(dim, L, md)
    da = dkt.DA(c, lv, dim, order=1, max_depth=md, sorted_tree=False)
    A = dkt.Matrix(da, op=dkt.OP_LAPMASS)
    import torch
    x = torch.zeros(da.n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    lib = dkt.load()
    rc = lib.dkt_fematrix_matvec_noalloc(A._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 1.0, None)
    assert rc == dkt.E_ARG
    assert b"exceed" in lib.dkt_last_error()
