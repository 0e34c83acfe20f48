"""Pin the CPU oracle against the reference's own outputs (golden fixtures).

The fixtures were produced by the unmodified reference sources
(tests/golden/make_golden.py).  Integer outputs must match bit for bit;
floating-point outputs within 1e-12 relative (2-norm) and the 1D reference
element operators within 1e-14.
"""
import glob
import os

import numpy as np
import pytest

import oracle_port as op
import trees

GOLDEN = sorted(glob.glob(os.path.join(os.path.dirname(__file__), "golden", "*.npz")))
MORTON = [g for g in GOLDEN if os.path.basename(g).startswith("morton_")]
HILBERT = [g for g in GOLDEN if os.path.basename(g).startswith("hilbert_")]


def _rel(a, b):
    nb = np.linalg.norm(b)
    return np.linalg.norm(a - b) / (nb if nb > 0 else 1.0)


def _oracle_tree(g):
    dim = int(g["dim"])
    if int(g["in_kind"]) == 0:
        return op.tree_balance(g["in_coords"], dim)
    if int(g["in_kind"]) == 3:
        # DA(func): the oracle has no function2Octree; it re-sorts the
        # reference's tree (shuffled) and takes the DA from there
        perm = np.random.default_rng(0).permutation(g["tree_levels"].size)
        return op.tree_sort(g["tree_coords"][perm], g["tree_levels"][perm], dim)
    return op.tree_sort(g["in_coords"], g["in_levels"], dim)


@pytest.mark.parametrize("path", MORTON, ids=[os.path.basename(p)[:-4] for p in MORTON])
def test_oracle_matches_reference(path):
    g = np.load(path)
    dim, md = int(g["dim"]), int(g["md"])
    op.set_curve(dim, md)
    tc, tl = _oracle_tree(g)
    assert np.array_equal(tc, g["tree_coords"]) and np.array_equal(tl, g["tree_levels"])
    da = op.DA(tc, tl, dim, int(g["order"]), int(g["op"]))
    assert np.array_equal(da.node_coords, g["node_coords"])
    assert np.array_equal(da.node_levels, g["node_levels"])
    assert np.array_equal(da.bdry, g["bdry"])
    re = da.refel()
    for k in ("ip0", "ip1", "Q1d", "Dg", "W"):
        assert np.max(np.abs(re[k] - g[k])) < 1e-14, k
    assert _rel(da.matvec(g["x"]), g["y"]) <= 1e-12
    assert _rel(da.matvec_raw(g["x"]), g["y_raw"]) <= 1e-12


@pytest.mark.parametrize("path", HILBERT, ids=[os.path.basename(p)[:-4] for p in HILBERT])
def test_hilbert_tables_reproduce_reference(path):
    """The library's own harmonious-Hilbert rotation tables (generated from
    Haverkort's refinement rule, not taken from the reference), loaded into
    the oracle, reproduce the reference's Hilbert-ordered trees, DA node
    order and products."""
    import __graft_entry__ as ge
    dkt = ge.load_package()
    g = np.load(path)
    dim, md = int(g["dim"]), int(g["md"])
    rot, ht = dkt.curve_tables(dkt.CURVE_HILBERT, dim)
    assert ht.size >> dim == {2: 4, 3: 24, 4: 192}[dim]
    op.set_curve(dim, md, rot, ht)
    try:
        tc, tl = _oracle_tree(g)
        assert np.array_equal(tc, g["tree_coords"]) and np.array_equal(tl, g["tree_levels"])
        da = op.DA(tc, tl, dim, int(g["order"]), int(g["op"]))
        assert np.array_equal(da.node_coords, g["node_coords"])
        assert np.array_equal(da.node_levels, g["node_levels"])
        assert np.array_equal(da.bdry, g["bdry"])
        assert _rel(da.matvec(g["x"]), g["y"]) <= 1e-12
    finally:
        op.set_curve(dim, md)


@pytest.mark.parametrize("ex,dim,L,order", [
    ("1", 2, 5, 1), ("1", 3, 4, 1), ("1", 2, 4, 2), ("2", 2, 4, 1), ("2", 3, 3, 2), ("3", 2, 4, 1), ("3", 3, 4, 1),
    ("1", 4, 3, 1), ("3", 4, 3, 1)])
def test_known_node_counts(ex, dim, L, order):
    """Closed-form CG node counts (test/testCountCGNodes.cpp:130-174)."""
    md = 8
    op.set_curve(dim, md)
    c, lv = getattr(trees, "example" + ex)(dim, L, md)
    c, lv = op.tree_sort(c, lv, dim)
    da = op.DA(c, lv, dim, order, 0)
    assert da.n == getattr(trees, f"example{ex}_num_points")(dim, L, order)


@pytest.mark.parametrize("dim,L", [(2, 3), (3, 3), (4, 2)])
def test_identity_uniform_intersection_degree(dim, L):
    """Identity eleOp, all-ones input, uniform grid: each node receives 2^k with
    k the number of axes along which it is interior (test/testMatvec.cpp:254-264)."""
    md = 6
    op.set_curve(dim, md)
    c, lv = op.tree_sort(*trees.example2(dim, L, md), dim)
    da = op.DA(c, lv, dim, 1, 0)
    y = da.matvec(np.ones(da.n))
    top = 1 << md
    k = np.sum((da.node_coords != 0) & (da.node_coords != top), axis=1)
    assert np.array_equal(y, 2.0 ** k)


def test_identity_adaptive_2d_linear():
    """Adaptive 2D linear: every node receives 2^k or 5 (test/testMatvec.cpp:373)."""
    dim, md, L = 2, 6, 4
    op.set_curve(dim, md)
    c, lv = op.tree_sort(*trees.example1(dim, L, md), dim)
    da = op.DA(c, lv, dim, 1, 0)
    y = da.matvec(np.ones(da.n))
    top = 1 << md
    grid = (1 << (md - da.node_levels.astype(np.int64)))[:, None] - 1
    k = dim - np.sum(((da.node_coords & grid) != 0) | ((da.node_coords % top) == 0), axis=1)
    assert np.all((np.abs(y - 2.0 ** k) < 1e-4) | (np.abs(y - 5.0) < 1e-4))


def test_no_stale_parent_reads_on_nondegenerate_meshes():
    """The static parent buffer is never read in a slot it did not refill
    (with nonzero interpolation weight) on the golden Morton meshes whose
    node spacing does not collapse.  The DA(func) meshes are left out: the 4D
    one does read stale slots (852 per product), and its fixture pins the
    emulation against the reference itself."""
    for path in MORTON:
        if "_f2o" in path:
            continue
        g = np.load(path)
        dim = int(g["dim"])
        op.set_curve(dim, int(g["md"]))
        da = op.DA(g["tree_coords"], g["tree_levels"], dim, int(g["order"]), int(g["op"]))
        da.matvec(g["x"])
        assert da.stats()["stale_reads"] == 0, path


CG = [g for g in GOLDEN if "_cg_" in os.path.basename(g)]


@pytest.mark.parametrize("path", CG, ids=[os.path.basename(p)[:-4] for p in CG])
def test_oracle_cgsolve_matches_reference(path):
    """HeatMat<3>::cgSolve restated in the oracle (no preconditioner,
    relative L-infinity stop) against the reference's own run on the same
    mesh and right-hand side: the same iteration count and final residual,
    and the solution within 1e-12 relative."""
    import __graft_entry__ as ge
    g = np.load(path)
    dim, md = int(g["dim"]), int(g["md"])
    if os.path.basename(path).startswith("hilbert_"):
        dkt = ge.load_package()
        op.set_curve(dim, md, *dkt.curve_tables(dkt.CURVE_HILBERT, dim))
    else:
        op.set_curve(dim, md)
    try:
        da = op.DA(g["tree_coords"], g["tree_levels"], dim, int(g["order"]), int(g["op"]))
        assert np.array_equal(da.node_coords, g["node_coords"])
        x, it, res, status = da.cg_ref(g["cg_b"], max_iter=int(g["cg_max_iter"]), tol=float(g["cg_tol"]))
        assert status == int(g["cg_status"]) == 0
        assert it == int(g["cg_iters"])
        assert abs(res - float(g["cg_resid"])) <= 1e-6 * float(g["cg_resid"])
        assert _rel(x, g["cg_x"]) <= 1e-12
    finally:
        op.set_curve(dim, md)
