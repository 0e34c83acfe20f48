"""Hanging-node slots of the tiled Q1 kernel (dkt_plan_set_hanging_slots).

With slots, the hanging leaves of a tile that meet at one hanging point read
one shared slot (the mean of the parent face's corners), and each slot's sum
goes to the face's corners once per tile; the reference traversal's rule that
the shared parent corner gets nothing from the leaf is kept by taking the
leaf's share back at its rank-0 node.  Hanging leaves that cannot use slots
(those reading stale parent slots, among others) run in the per-leaf kernel,
and with slots off every hanging leaf does.  The two forms round differently
only where a node's unit differs from the tile's: the products agree to
1e-13 relative, and both stay as close to the dense FP64 kernel as before.
The binary32 product stays within its 2e-6 bound of the FP64 product."""
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


def _meshes(dkt):
    pts = dkt.gaussian_points(3000, 3, 9, seed=4)
    tc, tl = dkt.tree_from_points(pts, 3, 9)
    yield "gauss3d", dkt.DA(tc, tl, 3, order=1, max_depth=9)
    pts = dkt.gaussian_points(2000, 2, 10, seed=5)
    tc, tl = dkt.tree_from_points(pts, 2, 10)
    yield "gauss2d", dkt.DA(tc, tl, 2, order=1, max_depth=10)
    tc, tl = dkt.moving_ball_tree(max_depth=10, level=5, device=True)
    yield "ball4d", dkt.DA(tc, tl, 4, order=1, max_depth=10)


def _product(A, x):
    import torch
    y = torch.full_like(x, float("nan"))
    A.matvec(x, y)
    torch.cuda.synchronize()
    return y.cpu().numpy()


@pytest.mark.parametrize("traversal", ["reference", "conforming"])
def test_slots_match_the_per_leaf_product(dkt, traversal):
    import torch
    trav = dkt.TRAVERSAL_REFERENCE if traversal == "reference" else dkt.TRAVERSAL_CONFORMING
    for name, da in _meshes(dkt):
        for op in (dkt.OP_LAPMASS, dkt.OP_LAPLACE):
            A = dkt.Matrix(da, op=op, traversal=trav)
            st = A.stats()
            assert st["hanging_leaves"] > 0, name
            assert st["hanging_slots"] > 0 and st["slot_reading_leaves"] > 0, (name, st)
            if name != "ball4d":
                # 2:1-balanced 2D / 3D meshes: every hanging leaf reads slots
                assert st["slot_reading_leaves"] == st["hanging_leaves"], (name, st)
            else:
                assert st["slot_reading_leaves"] >= 0.6 * st["hanging_leaves"], (name, st)
            x = torch.from_numpy(dkt.uniform_pm1(7, da.n)).cuda()
            y_on = _product(A, x)
            A.set_hanging_slots(False)
            st_off = A.stats()
            assert st_off["hanging_slots"] == 0 and st_off["slot_reading_leaves"] == 0
            y_off = _product(A, x)
            A.set_hanging_slots(True)
            y_on2 = _product(A, x)
            assert np.all(np.isfinite(y_on)), name
            nrm = np.linalg.norm(y_off)
            assert np.linalg.norm(y_on - y_off) <= 1e-13 * nrm, (name, traversal, op)
            assert np.array_equal(y_on, y_on2), name
            A.set_arithmetic(dkt.ARITH_FP64)
            y_dense = _product(A, x)
            A.set_arithmetic(dkt.ARITH_AUTO)
            assert np.linalg.norm(y_on - y_dense) <= 1e-13 * np.linalg.norm(y_dense), (name, traversal, op)
            for T in ((64, 128) if name == "ball4d" else (128, 512)):
                A.set_tile(T)
                yt = _product(A, x)
                err = np.linalg.norm(yt - y_on) / np.linalg.norm(y_on)
                assert err <= 1e-13, (name, T, err)
            A.set_tile(256)


@pytest.mark.parametrize("traversal", ["reference", "conforming"])
def test_slots_binary32_product(dkt, traversal):
    import torch
    trav = dkt.TRAVERSAL_REFERENCE if traversal == "reference" else dkt.TRAVERSAL_CONFORMING
    for name, da in _meshes(dkt):
        A = dkt.Matrix(da, op=dkt.OP_LAPLACE, traversal=trav)
        if A.stats()["stale_slots"] > 0:
            continue
        x = dkt.uniform_pm1(3, da.n)
        y64 = torch.empty(da.n, dtype=torch.float64, device="cuda")
        A.matvec(torch.from_numpy(x).cuda(), y64)
        b = y64.cpu().numpy()
        for on in (True, False):
            A.set_hanging_slots(on)
            y32 = torch.empty(da.n, dtype=torch.float32, device="cuda")
            A.matvec_f32(torch.from_numpy(x.astype(np.float32)).cuda(), y32)
            a = y32.double().cpu().numpy()
            assert np.linalg.norm(a - b) / np.linalg.norm(b) <= 2e-6, (name, traversal, on)


def test_slots_in_a_batch(dkt):
    """A batch keeps each plan's slots (tile-local) with moved offsets."""
    import torch
    mats, xs = [], []
    for k in range(3):
        pts = dkt.cluster_points(600 + 300 * k, 3, 9, seed=k)
        tc, tl = dkt.tree_from_points(pts, 3, 9)
        da = dkt.DA(tc, tl, 3, order=1, max_depth=9)
        mats.append(dkt.Matrix(da, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING))
        xs.append(dkt.uniform_pm1(11 + k, da.n))
    B = dkt.Matrix.batch(mats)
    assert B.stats()["hanging_slots"] == sum(m.stats()["hanging_slots"] for m in mats)
    xb = torch.from_numpy(np.concatenate(xs)).cuda()
    yb = _product(B, xb)
    off = B.mesh_offsets()
    for k, m in enumerate(mats):
        yk = _product(m, torch.from_numpy(xs[k]).cuda())
        assert np.linalg.norm(yb[off[k]:off[k + 1]] - yk) <= 1e-12 * np.linalg.norm(yk), k
