"""Properties of the trees that feed the matvec path, as the reference's own
tests state them: complete, 2:1 balanced over all 3^dim - 1 neighbours
(test/testTreeBalancing.cpp:607-677), sorting preserves the cells
(test/testTreeSort.cpp:85-110), and consecutive cells of a uniform grid in
Hilbert order are face neighbours (test/testHCurveTable.cpp:68-155).  The
host builders and the oracle run on the CPU; the device builders are checked
in the tests marked gpu."""
import itertools

import numpy as np
import pytest

import __graft_entry__ as ge
import oracle_port as orc


@pytest.fixture(scope="module")
def dkt():
    return ge.load_package()


def _keys(coords, dim, md):
    k = np.zeros(coords.shape[0], np.int64)
    for d in range(dim):
        k |= coords[:, d].astype(np.int64) << (d * md)
    return k


def max_level_jump(coords, levels, dim, md):
    """Largest level difference between a leaf and any leaf touching it
    (faces, edges or corners).  A finer neighbour two or more levels down is
    found from its own side: the point just outside it towards the coarse
    leaf lies in the coarse leaf."""
    coords = np.asarray(coords, np.int64).reshape(-1, dim)
    levels = np.asarray(levels, np.int64)
    top = 1 << md
    by_level = {l: np.sort(_keys(coords[levels == l], dim, md)) for l in np.unique(levels)}
    length = (1 << (md - levels))[:, None]
    worst = 0
    for delta in itertools.product((-1, 0, 1), repeat=dim):
        if not any(delta):
            continue
        p = coords.copy()
        for d, s in enumerate(delta):
            if s == 1:
                p[:, d] += length[:, 0]
            elif s == -1:
                p[:, d] -= 1
        inside = np.all((p >= 0) & (p < top), axis=1)
        found = np.full(coords.shape[0], -1, np.int64)
        for l, keys in by_level.items():
            a = p & ~np.int64((1 << (md - l)) - 1)
            k = _keys(a, dim, md)
            pos = np.clip(np.searchsorted(keys, k), 0, max(len(keys) - 1, 0))
            hit = inside & (found < 0) & (len(keys) > 0) & (keys[pos] == k)
            found[hit] = l
        assert np.all(found[inside] >= 0), "a point inside the domain lies in no leaf"
        worst = max(worst, int(np.max(np.abs(found[inside] - levels[inside]), initial=0)))
    return worst


def assert_complete_balanced(coords, levels, dim, md):
    levels = np.asarray(levels)
    vol = np.sum(2.0 ** (-dim * levels.astype(np.float64)))
    assert abs(vol - 1.0) < 1e-12
    assert len(set(map(tuple, np.concatenate([np.asarray(coords, np.int64).reshape(-1, dim),
                                               levels[:, None].astype(np.int64)], 1)))) == len(levels)
    assert max_level_jump(coords, levels, dim, md) <= 1


@pytest.mark.parametrize("dim,n,md,max_pts", [(2, 2000, 10, 1), (3, 3000, 8, 1), (3, 3000, 8, 5), (4, 300, 6, 1)])
def test_host_points_tree_complete_and_balanced(dkt, dim, n, md, max_pts):
    pts = dkt.gaussian_points(n, dim, md, seed=2)
    c, l = dkt.tree_from_points(pts, dim, md, max_pts=max_pts)
    assert_complete_balanced(c, l, dim, md)


def test_host_moving_ball_and_sphere_complete_and_balanced(dkt):
    c, l = dkt.moving_ball_tree(max_depth=6, level=4)
    assert_complete_balanced(c, l, 4, 6)
    c, l = dkt.sphere_shell_tree(3, 8, 5, (0.4, 0.5, 0.55), 0.3, device=False)
    assert_complete_balanced(c, l, 3, 8)


def test_checker_finds_an_unbalanced_tree():
    """The checker itself: a 2D tree with a level-3 cell beside a level-1 cell."""
    md = 4
    cells = [((8, 0), 1), ((0, 8), 1), ((8, 8), 1)]   # three level-1 quadrants
    # the lower-left quadrant split to level 2, its lower-right child to level 3
    cells += [((0, 0), 2), ((0, 4), 2), ((4, 4), 2)]
    cells += [((4, 0), 3), ((6, 0), 3), ((4, 2), 3), ((6, 2), 3)]
    c = np.array([a for a, _ in cells], np.uint32)
    l = np.array([lv for _, lv in cells], np.uint8)
    assert abs(np.sum(2.0 ** (-2 * l.astype(np.float64))) - 1.0) < 1e-12
    assert max_level_jump(c, l, 2, md) == 2


@pytest.mark.parametrize("dim,n,md", [(2, 500, 8), (3, 800, 7), (4, 200, 5)])
def test_sort_preserves_cells(dkt, dim, n, md):
    """locTreeSort of a shuffled tree with repeated cells keeps every cell
    (count and multiset), for both curves."""
    pts = dkt.gaussian_points(n, dim, md, seed=4)
    c, l = dkt.tree_from_points(pts, dim, md)
    idx = np.random.default_rng(1).integers(0, len(l), len(l) + len(l) // 3)
    c, l = c[idx], l[idx]
    for curve in (dkt.CURVE_MORTON, dkt.CURVE_HILBERT):
        if curve == dkt.CURVE_HILBERT:
            rot, ht = dkt.curve_tables(curve, dim)
            orc.set_curve(dim, md, rot, ht)
        else:
            orc.set_curve(dim, md)
        try:
            sc, sl = orc.tree_sort(c, l, dim)
        finally:
            orc.set_curve(dim, md)
        assert len(sl) == len(l)
        key = lambda cc, ll: sorted(map(tuple, np.concatenate([cc.astype(np.int64), ll[:, None].astype(np.int64)], 1)))
        assert key(sc, sl) == key(c, l)


@pytest.mark.parametrize("dim,L", [(2, 5), (3, 3), (4, 2)])
def test_hilbert_order_is_face_continuous(dkt, dim, L):
    """Uniform level-L grid sorted along the library's Hilbert curve:
    consecutive cells share a face (differ by one cell in one coordinate)."""
    md = L + 1
    n1 = 1 << L
    grid = np.array(list(itertools.product(range(n1), repeat=dim)), np.uint32) << np.uint32(md - L)
    lv = np.full(len(grid), L, np.uint8)
    rot, ht = dkt.curve_tables(dkt.CURVE_HILBERT, dim)
    orc.set_curve(dim, md, rot, ht)
    try:
        sc, _ = orc.tree_sort(grid[np.random.default_rng(0).permutation(len(grid))], lv, dim)
    finally:
        orc.set_curve(dim, md)
    step = np.abs(np.diff(sc.astype(np.int64), axis=0)) >> (md - L)
    assert np.all(step.sum(axis=1) == 1)
    # and Morton order is not (a check that the test can fail)
    orc.set_curve(dim, md)
    mc, _ = orc.tree_sort(grid, lv, dim)
    mstep = np.abs(np.diff(mc.astype(np.int64), axis=0)) >> (md - L)
    assert not np.all(mstep.sum(axis=1) == 1)


@pytest.mark.gpu
def test_device_trees_complete_and_balanced(dkt):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    for dim, n, md in ((2, 3000, 12), (3, 20000, 10), (4, 800, 8)):
        c, l = dkt.tree_from_points(dkt.gaussian_points(n, dim, md, seed=9), dim, md, device=True)
        assert_complete_balanced(c, l, dim, md)
    c, l = dkt.moving_ball_tree(max_depth=8, level=5, device=True)
    assert_complete_balanced(c, l, 4, 8)
    for dim in (2, 3, 4):
        c, l = dkt.sphere_shell_tree(dim, 9, 5, (0.5,) * dim, 0.3)
        assert_complete_balanced(c, l, dim, 9)
