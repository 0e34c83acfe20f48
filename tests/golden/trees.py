"""Analytic test meshes and point clouds used by the parity tests.

The three analytic trees restate the known-answer meshes of the reference's
tests (test/testAdaptiveExamples.h): Example1 refines towards the domain
centre, Example2 is uniform, Example3 refines a fringe along the domain
boundary.  Each comes with the closed-form count of CG nodes the reference
test checks (test/testCountCGNodes.cpp:130-174).  Trees are returned in
Morton child order (the order the reference generators emit); callers sort.
"""
import numpy as np


def _child(anchor, level, ch, dim, md):
    ln = 1 << (md - level - 1)
    return tuple(anchor[d] | (ln if (ch >> d) & 1 else 0) for d in range(dim)), level + 1


def example1(dim, end_level, md):
    """Minimal balanced tree with 2^dim level-end_level cells at the centre."""
    nc = 1 << dim
    out = []

    def corner(anchor, level, ch):
        if level >= end_level:
            out.append((anchor, level))
            return
        for other in range(nc):
            if other != ch:
                out.append(_child(anchor, level, other, dim, md))
        a, l = _child(anchor, level, ch, dim, md)
        corner(a, l, ch)

    root = (tuple([0] * dim), 0)
    for ch in range(nc):
        a, l = _child(root[0], 0, ch, dim, md)
        corner(a, l, nc - 1 - ch)
    return _pack(out, dim)


def example1_num_points(dim, end_level, order):
    return (end_level - 2) * ((4 * order - 1) ** dim - (2 * order - 1) ** dim) + (4 * order + 1) ** dim


def example2(dim, end_level, md):
    """Uniform grid of level end_level."""
    n = 1 << end_level
    idx = np.indices([n] * dim).reshape(dim, -1).T[:, ::-1]
    coords = (idx.astype(np.uint32) << np.uint32(md - end_level))
    return coords, np.full(coords.shape[0], end_level, np.uint8)


def example2_num_points(dim, end_level, order):
    return ((1 << end_level) * order + 1) ** dim


def example3(dim, end_level, md):
    """Minimal balanced tree with a level-end_level fringe on the boundary."""
    nc = 1 << dim
    top = 1 << md
    out = []

    def touching(anchor, level):
        ln = 1 << (md - level)
        return any(a == 0 or a + ln == top for a in anchor)

    def sub(anchor, level):
        if level >= end_level:
            out.append((anchor, level))
            return
        for ch in range(nc):
            a, l = _child(anchor, level, ch, dim, md)
            if touching(a, l):
                sub(a, l)
            else:
                out.append((a, l))

    for ch in range(nc):
        a, l = _child(tuple([0] * dim), 0, ch, dim, md)
        sub(a, l)
    return _pack(out, dim)


def example3_num_points(dim, end_level, order):
    total = example2_num_points(dim, end_level, order)
    for lv in range(2, end_level):
        total += ((2 ** lv - 2) * order + 1) ** dim
        total -= ((2 ** (lv + 1) - 4) * order + 1) ** dim
    return total


def _pack(cells, dim):
    coords = np.array([c[0] for c in cells], dtype=np.uint32).reshape(-1, dim)
    levels = np.array([c[1] for c in cells], dtype=np.uint8)
    return coords, levels


def gaussian_points(n, dim, md, mean=0.5, sd=0.1, seed=0):
    """Isotropic Gaussian cloud clipped to the unit cube, as level-md points."""
    rng = np.random.default_rng(seed)
    x = rng.normal(mean, sd, size=(n, dim))
    x = np.clip(x, 0.0, 1.0 - 2.0 ** -md)
    return np.floor(x * (1 << md)).astype(np.uint32)
