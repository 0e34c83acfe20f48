"""A mesh in parts on one GPU (dendro-kt_gb300/partition.py with
dkt_plan_create_part): the ghost read, the parts' own products on their
ghosted layouts, and the ghost accumulate give the one-part fem::matvec, to
the fixed-point round-off of the parts' own units (1e-12 relative).  A plan
that reads stale slots of the reference's static parent buffer is refused."""
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
    da3 = dkt.DA(tc, tl, 3, order=1, max_depth=9)
    yield "gauss3d_q1_lapmass", dkt.Matrix(da3, op=dkt.OP_LAPMASS), da3
    da3q = dkt.DA(tc << np.uint32(1), tl, 3, order=2, max_depth=10)
    yield "gauss3d_q2_lapmass", dkt.Matrix(da3q, op=dkt.OP_LAPMASS), da3q
    tc, tl = dkt.moving_ball_tree(max_depth=10, level=5, device=True)
    da4 = dkt.DA(tc, tl, 4, order=1, max_depth=10)
    yield "ball4d_q1_conforming", dkt.Matrix(da4, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING), da4


@pytest.mark.parametrize("nparts", [2, 3, 4])
def test_parts_reproduce_the_one_part_product(dkt, nparts):
    import torch
    for name, A, da in _meshes(dkt):
        assert A.stats()["stale_slots"] == 0, name
        x = torch.from_numpy(dkt.uniform_pm1(5, da.n)).cuda()
        y = torch.empty_like(x)
        A.matvec_raw(x, y)
        P = dkt.partition.PartitionedMatrix(A, nparts)
        owned = np.concatenate([p["nodes"][dkt.partition.owned_slice(p)] for p in P.parts])
        assert np.array_equal(np.sort(owned), np.arange(da.n)), name
        assert sum(p["n_pre"] + p["n_post"] for p in P.parts) > 0, name      # there are ghosts
        yp = torch.full_like(x, float("nan"))
        P.matvec_raw(x, yp)
        torch.cuda.synchronize()
        a, b = yp.cpu().numpy(), y.cpu().numpy()
        err = np.linalg.norm(a - b) / np.linalg.norm(b)
        assert err <= 1e-12, (name, nparts, err)


def test_stale_reading_plan_is_not_partitioned(dkt):
    tc, tl = dkt.moving_ball_tree(max_depth=10, level=5, device=True)
    da = dkt.DA(tc, tl, 4, order=1, max_depth=10)
    A = dkt.Matrix(da, op=dkt.OP_LAPMASS)
    assert A.stats()["stale_slots"] > 0
    with pytest.raises(dkt.DktError) as e:
        dkt.partition.PartitionedMatrix(A, 2)
    assert e.value.code == dkt.E_UNSUP
