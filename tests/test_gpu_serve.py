"""The serving loop: concurrent requests of different dimension give the
same solutions as the same requests served one at a time (within the
solver tolerance), every solution has relative residual <= 1e-10 under the
FP64 product, and the admission budget serialises requests that do not fit
together."""
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


def _requests(dkt):
    reqs = []
    specs = [(2, 7, (0.4, 0.55), 0.3), (3, 5, (0.5, 0.45, 0.5), 0.25), (4, 4, (0.5, 0.5, 0.5, 0.5), 0.3),
             (3, 6, (0.45, 0.5, 0.55), 0.3), (2, 8, (0.5, 0.5), 0.2), (4, 3, (0.4, 0.5, 0.5, 0.6), 0.25)]
    for k, (dim, level, ctr, rad) in enumerate(specs):
        c, l = dkt.sphere_shell_tree(dim, 10, level, ctr, rad)
        reqs.append((dim, c, l, 100 + k))
    return reqs


def _residual(dkt, dim, c, l, seed, x):
    import torch
    da = dkt.DA(c, l, dim, order=1, max_depth=10)
    A = dkt.Matrix(da, op=dkt.OP_LAPLACE, traversal=dkt.TRAVERSAL_CONFORMING)
    b = dkt.uniform_pm1(seed, da.n)
    b[da.boundary_ids()] = 0.0
    xd = torch.from_numpy(x).cuda()
    y = torch.empty_like(xd)
    A.matvec(xd, y)
    return np.linalg.norm(b - y.cpu().numpy()) / np.linalg.norm(b)


def test_served_results_same_alone_and_in_the_mix(dkt):
    reqs = _requests(dkt)
    alone = []
    srv = dkt.Server(workers=1, budget_bytes=1.0)        # one request at a time
    for dim, c, l, seed in reqs:
        alone.append(srv.wait(srv.submit(c, l, dim, 10, seed)))
    srv.close()
    srv = dkt.Server(workers=4, budget_bytes=64e9)
    tickets = [srv.submit(c, l, dim, 10, seed) for dim, c, l, seed in reqs]
    mix = [srv.wait(t) for t in tickets]
    srv.close()
    for (dim, c, l, seed), a, m in zip(reqs, alone, mix):
        assert a["rc"] == 0 and m["rc"] == 0
        assert a["relres"] <= 1e-10 and m["relres"] <= 1e-10
        assert np.linalg.norm(a["x"] - m["x"]) <= 1e-6 * np.linalg.norm(a["x"]), dim
        assert _residual(dkt, dim, c, l, seed, m["x"]) <= 1e-10
    # the mix ran concurrently: some service intervals overlap
    iv = sorted((m["t_start"], m["t_done"]) for m in mix)
    assert any(iv[k + 1][0] < iv[k][1] for k in range(len(iv) - 1))


def test_budget_serialises(dkt):
    reqs = _requests(dkt)[:4]
    srv = dkt.Server(workers=4, budget_bytes=1.0)
    tickets = [srv.submit(c, l, dim, 10, seed) for dim, c, l, seed in reqs]
    res = [srv.wait(t, solution=False) for t in tickets]
    srv.close()
    iv = sorted((r["t_start"], r["t_done"]) for r in res)
    assert all(iv[k + 1][0] >= iv[k][1] for k in range(len(iv) - 1))
    assert all(r["device_bytes"] > 0 for r in res)
