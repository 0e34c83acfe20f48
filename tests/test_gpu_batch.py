"""Batches of independent meshes as one block-diagonal plan: the batched
product equals the products of the meshes one by one, and the batched
solvers converge every mesh to 1e-10 on its own, to the same solutions as
solving the meshes one at a time."""
import numpy as np
import pytest

import __graft_entry__ as ge

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def dkt():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return ge.load_package()


def _meshes(dkt, sizes, dim=3, md=10, order=1):
    out = []
    for k, n in enumerate(sizes):
        # order 2: the tree one level coarser in coordinates, so Q2 node spacing stays integral
        gmd = md - 1 if order == 2 else md
        tc, tl = dkt.tree_from_points(dkt.cluster_points(n, dim, gmd, seed=k), dim, gmd)
        if order == 2:
            tc = tc << np.uint32(1)
        out.append(dkt.DA(tc, tl, dim, order=order, max_depth=md))
    return out


def _mv(A, x):
    import torch
    xd = torch.from_numpy(np.ascontiguousarray(x)).cuda()
    yd = torch.empty_like(xd)
    A.matvec(xd, yd)
    return yd.cpu().numpy()


@pytest.mark.parametrize("order", [1, 2])
def test_batched_product_equals_single_products(dkt, order):
    das = _meshes(dkt, [300, 1200, 50, 2500], order=order)
    mats = [dkt.Matrix(d, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING) for d in das]
    B = dkt.Matrix.batch(mats)
    off = B.mesh_offsets()
    assert B.num_meshes() == 4 and off[-1] == sum(d.n for d in das) == B.n
    xs = [dkt.uniform_pm1(10 + k, d.n) for k, d in enumerate(das)]
    yb = _mv(B, np.concatenate(xs))
    for k, (A, x) in enumerate(zip(mats, xs)):
        y = _mv(A, x)
        seg = yb[off[k]:off[k + 1]]
        assert np.linalg.norm(seg - y) <= 1e-12 * np.linalg.norm(y), k


@pytest.mark.parametrize("precision,order", [(0, 1), (1, 1), (0, 2), (1, 2)])
def test_batched_pcg_per_mesh_convergence(dkt, precision, order):
    import torch
    das = _meshes(dkt, [400, 2000, 100, 3000, 800], order=order)
    mats = [dkt.Matrix(d, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING) for d in das]
    B = dkt.Matrix.batch(mats)
    off = B.mesh_offsets()
    bs = []
    for k, d in enumerate(das):
        b = dkt.uniform_pm1(20 + k, d.n)
        b[d.boundary_ids()] = 0.0
        bs.append(b)
    bd = torch.from_numpy(np.concatenate(bs)).cuda()
    xd = torch.zeros_like(bd)
    it, ref, rr, ok = B.pcg(bd, xd, precision=precision, tol=1e-10)
    assert ok and len(it) == 5 and np.all(rr <= 1e-10), (it, ref, rr)
    if precision == 1:
        # well-conditioned meshes at different stages of convergence at each
        # reliable update: every one stays in the binary32 sequence
        assert B.stats()["fp64_finishes"] == 0 and np.all(ref >= 1), ref
    x = xd.cpu().numpy()
    for k, (A, d) in enumerate(zip(mats, das)):
        xk = x[off[k]:off[k + 1]]
        r = bs[k] - _mv(A, xk)
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(bs[k]), k
        bk = torch.from_numpy(bs[k]).cuda()
        x1 = torch.zeros_like(bk)
        it1, ref1, rr1, ok1 = A.pcg(bk, x1, precision=precision, tol=1e-10)
        assert ok1
        x1 = x1.cpu().numpy()
        assert np.linalg.norm(xk - x1) <= 1e-6 * np.linalg.norm(x1), k
        if precision == 0:
            # Q1 products are exact integers; the Q2 product sums with FP64
            # atomics, whose order varies, so its iteration counts may differ a little
            slack = 2 if order == 1 else max(2, it1 // 100)
            assert abs(int(it[k]) - it1) <= slack, (k, it[k], it1)


def test_autotune_keeps_result(dkt):
    import torch
    (d,) = _meshes(dkt, [5000])
    A = dkt.Matrix(d, op=dkt.OP_LAPMASS)
    x = dkt.uniform_pm1(3, d.n)
    y0 = _mv(A, x)
    T, persist, ms, times = A.autotune()
    assert T in (0, 128, 256, 512) and ms > 0 and ms == min(t for t in times if t > 0)
    y1 = _mv(A, x)
    # another tile size rounds in other fixed-point units: a few units apart
    assert np.linalg.norm(y1 - y0) <= 1e-13 * np.linalg.norm(y0)
    # the binary32 product of the mixed solver (a conforming plan)
    C = dkt.Matrix(d, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING)
    T32, p32, ms32, t32 = C.autotune(arith=1)
    assert ms32 > 0 and T32 in (0, 128, 256, 512) and ms32 == min(t for t in t32 if t > 0)


@pytest.mark.parametrize("precision", [0, 1])
def test_batched_pcg_tiles_spanning_small_meshes(dkt, precision):
    """Forty small 2D meshes (7-60 leaves), re-tiled over the whole batch so
    that each tile covers several of them; three in four have a zero
    right-hand side and converge at once.  A tile whose first and last meshes
    are done still holds live meshes between them, whose products must go on;
    the zero meshes keep x = 0."""
    import torch
    das = []
    for k in range(40):
        c, l = dkt.tree_from_points(dkt.cluster_points(3, 2, 8, seed=k), 2, 8)
        das.append(dkt.DA(c, l, 2, order=1, max_depth=8))
    mats = [dkt.Matrix(d, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING) for d in das]
    B = dkt.Matrix.batch(mats)
    B.set_tile(256)
    off = B.mesh_offsets()
    bs = []
    for k, d in enumerate(das):
        b = dkt.uniform_pm1(50 + k, d.n) if k % 4 == 1 else np.zeros(d.n)
        b[d.boundary_ids()] = 0.0
        bs.append(b)
    bd = torch.from_numpy(np.concatenate(bs)).cuda()
    xd = torch.zeros_like(bd)
    it, ref, rr, ok = B.pcg(bd, xd, precision=precision, tol=1e-10)
    assert ok and np.all(rr <= 1e-10), (it, rr)
    x = xd.cpu().numpy()
    for k, (A, d) in enumerate(zip(mats, das)):
        xk = x[off[k]:off[k + 1]]
        if k % 4 != 1:
            assert not np.any(xk), k
            assert it[k] == 0, (k, it[k])
            continue
        r = bs[k] - _mv(A, xk)
        assert np.linalg.norm(r) <= 1e-10 * np.linalg.norm(bs[k]), k
