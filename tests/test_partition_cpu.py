"""The partitioned-mesh host logic (dendro-kt_gb300/partition.py) on the CPU:
SFC partition, node ownership, the ghosted [pre | owned | post] layout, the
send/receive lists and the ghost read / ghost accumulate.

A toy traversal stands in for a plan's flattened one: a 2D grid of Q1 cells
(node ids row-major) whose element operator is a dense random 4 x 4 matrix
per cell, plus "hanging" records that add a weighted copy of a cell's own
values into parent nodes elsewhere -- linear, and touching nodes outside the
cell's own part, as the hanging transposes do.  The partitioned product
(parts in one process, and parts on two gloo ranks) must equal the product
on the whole mesh to round-off."""
import os
import socket
import subprocess
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, REPO)


def _pkg():
    import __graft_entry__ as ge
    return ge.load_package()


def toy_mesh(m=9, seed=0):
    """e2n [m*m][4], hidx, p2n, per-cell matrices K, hanging weights W."""
    rng = np.random.default_rng(seed)
    nid = np.arange((m + 1) * (m + 1)).reshape(m + 1, m + 1)
    e2n = np.array([[nid[j, i], nid[j, i + 1], nid[j + 1, i], nid[j + 1, i + 1]] for j in range(m) for i in range(m)],
                   np.int32)
    n_leaf = e2n.shape[0]
    hidx = np.full(n_leaf, -1, np.int32)
    hanging = rng.choice(n_leaf, size=n_leaf // 4, replace=False)
    hanging.sort()
    hidx[hanging] = np.arange(hanging.size)
    p2n = rng.integers(0, (m + 1) * (m + 1), size=(hanging.size, 4)).astype(np.int32)
    p2n[rng.random(p2n.shape) < 0.25] = -1
    K = rng.standard_normal((n_leaf, 4, 4))
    W = rng.standard_normal((hanging.size, 4))
    return e2n, hidx, p2n, K, W, (m + 1) * (m + 1)


def local_product(e2n, hidx, p2n, K, W, x):
    """The toy operator on one traversal (whole mesh or one part, in its own
    node numbering)."""
    y = np.zeros_like(x)
    for e in range(e2n.shape[0]):
        np.add.at(y, e2n[e], K[e] @ x[e2n[e]])
        h = hidx[e]
        if h >= 0:
            ok = p2n[h] >= 0
            np.add.at(y, p2n[h][ok], (W[h] * x[e2n[e]])[ok])
    return y


def part_product(part, e2n, hidx, p2n, K, W, xl):
    b0, b1 = part["leaf_begin"], part["leaf_end"]
    nm = part["node_map"]
    le2n = nm[e2n[b0:b1]]
    hh = hidx[b0:b1]
    lp2n = np.where(p2n >= 0, nm[np.maximum(p2n, 0)], -1)
    return local_product(le2n, hh, lp2n, K[b0:b1], W, xl)


@pytest.mark.parametrize("nparts", [1, 2, 3, 5])
def test_partitioned_product_in_one_process(nparts):
    P = _pkg().partition
    e2n, hidx, p2n, K, W, n = toy_mesh()
    x = np.random.default_rng(1).standard_normal(n)
    y = local_product(e2n, hidx, p2n, K, W, x)
    parts = P.partition_maps(e2n, hidx, p2n, n, nparts)
    # every node owned once; local layouts [pre | owned | post]
    owned = np.concatenate([p["nodes"][P.owned_slice(p)] for p in parts])
    assert np.array_equal(np.sort(owned), np.arange(n))
    for p in parts:
        assert p["nodes"].size == p["n_pre"] + p["n_owned"] + p["n_post"]
        assert p["n_post"] == 0          # owners come first: ghosts of later owners do not occur
    xs = []
    for p in parts:
        v = np.zeros(p["nodes"].size)
        v[P.owned_slice(p)] = x[p["nodes"][P.owned_slice(p)]]
        xs.append(v)
    P.read_from_ghosts(parts, xs)
    for p, v in zip(parts, xs):
        assert np.array_equal(v, x[p["nodes"]])           # every ghost took its owner's value
    ys = [part_product(p, e2n, hidx, p2n, K, W, v) for p, v in zip(parts, xs)]
    P.write_to_ghosts_accumulate(parts, ys)
    yp = np.zeros(n)
    for p, v in zip(parts, ys):
        o = P.owned_slice(p)
        yp[p["nodes"][o]] = v[o]
        assert np.all(v[:p["n_pre"]] == 0) and np.all(v[o.stop:] == 0)
    assert np.linalg.norm(yp - y) <= 1e-13 * np.linalg.norm(y)


def _worker():
    import torch
    import torch.distributed as dist
    dist.init_process_group("gloo")
    rank, world = dist.get_rank(), dist.get_world_size()
    P = _pkg().partition
    e2n, hidx, p2n, K, W, n = toy_mesh()
    x = np.random.default_rng(1).standard_normal(n)
    parts = P.partition_maps(e2n, hidx, p2n, n, world)
    part = parts[rank]
    o = P.owned_slice(part)
    xl = torch.zeros(part["nodes"].size, dtype=torch.float64)
    xl[o] = torch.from_numpy(x[part["nodes"][o]])
    P.exchange_read(part, xl)
    assert np.array_equal(xl.numpy(), x[part["nodes"]])
    yl = torch.from_numpy(part_product(part, e2n, hidx, p2n, K, W, xl.numpy()))
    P.exchange_accumulate(part, yl)
    y = local_product(e2n, hidx, p2n, K, W, x)
    yo = y[part["nodes"][o]]
    err = np.linalg.norm(yl.numpy()[o] - yo) / max(np.linalg.norm(yo), 1e-300)
    assert err <= 1e-13, err
    dist.destroy_process_group()


def test_partitioned_product_on_two_gloo_ranks():
    """Two ranks, one part each, ghost values sent with torch.distributed
    (gloo) point-to-point calls."""
    pytest.importorskip("torch")
    with socket.socket() as sk:
        sk.bind(("127.0.0.1", 0))
        port = sk.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2", "--master-addr",
           "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, (r.stdout[-2000:], r.stderr[-3000:])


if __name__ == "__main__":      # one rank of test_partitioned_product_on_two_gloo_ranks
    _worker()
