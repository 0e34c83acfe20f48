"""Generate the golden fixtures in this folder from the reference build.

Runs only where the reference sources exist: builds oracle/ref (the
unmodified Dendro-KT sources + single-rank MPI stand-in) and records, for a
set of small meshes, the reference's own outputs:
  tree (SFC order), DA node list (coords, levels), boundary node ids,
  input vector x, feMatrix::matVec output y, raw fem::matvec output y_raw,
  and the RefElement 1D operators; for the driver's op 7 also
  HeatMat<3>::cgSolve from x = 0 on the HeatVec<3> right-hand side of x
  (status, final relative L-infinity residual, iterations, right-hand side,
  solution); and, under vtu/, io::vtk::oct2vtu of one 3D tree per curve
  (the driver's op 8: the tree and the written file's arrays).
Usage:  python tests/golden/make_golden.py [name-substring ...]
        (with arguments, only the fixtures whose names contain one of them)
"""
import os
import subprocess
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, HERE)
import refio  # noqa: E402
import trees  # noqa: E402

REF_DIR = os.path.join(REPO, "oracle", "_ref")


def build_ref():
    subprocess.run(["make", "-C", os.path.join(REPO, "oracle", "ref"), "-j2"], check=True)


CG_TOL, CG_MAX_ITER = 1e-10, 1000


def run_ref(curve, dim, md, order, op, coords, levels, kind, seed, x=None, interp_tol=None):
    exe = os.path.join(REF_DIR, "ref_driver_" + curve)
    inp = os.path.join("/tmp", "dkt_golden_in.bin")
    out = os.path.join("/tmp", "dkt_golden_out.bin")
    refio.write_input(inp, dim, md, order, op, coords, levels, input_kind=kind, seed=seed, x=x,
                      interp_tol=interp_tol, cg_tol=CG_TOL, cg_max_iter=CG_MAX_ITER)
    subprocess.run([exe, inp, out], check=True, stdout=subprocess.DEVNULL, stderr=subprocess.DEVNULL)
    return refio.read_output(out, dim)


def cases():
    # (name, curve, dim, md, order, op, source)
    out = []
    for curve in ("morton", "hilbert"):
        for dim in (2, 3, 4):
            md = 6 if dim < 4 else 5
            for order in (1, 2):
                lv = {2: (4, 3, 3), 3: (4, 3, 3), 4: (3, 2, 3)}[dim]
                if dim == 4 and order == 2:
                    lv = (3, 2, 2)
                for ex, L in zip(("ex1", "ex2", "ex3"), lv):
                    for op in (0, 2):
                        out.append((f"{curve}_d{dim}_p{order}_op{op}_{ex}L{L}", curve, dim, md, order, op, (ex, L)))
        # Gaussian point clouds through locTreeBalancing
        for dim, n, md in ((2, 200, 8), (3, 300, 8), (4, 40, 6)):
            out.append((f"{curve}_d{dim}_p1_op2_gauss{n}", curve, dim, md, 1, 2, ("gauss", n)))
            out.append((f"{curve}_d{dim}_p2_op2_gauss{n}", curve, dim, md + 1, 2, 2, ("gauss_shift", n)))
        out.append((f"{curve}_d3_p1_op1_gauss300", curve, 3, 8, 1, 1, ("gauss", 300)))
        out.append((f"{curve}_d3_p1_op1_ex1L4", curve, 3, 6, 1, 1, ("ex1", 4)))
        # feVector::computeVec of HeatVec<3> (a 3D operator in the reference).
        # Order 1 only: at order 2 the reference's output is NaN, since
        # basis::jacobiglq leaves the nodes unset for N == 2 under
        # WITH_BLAS_LAPACK (FEM/src/basis.cpp:175-186), so
        # RefElement::getElementSz() is 0 and HeatVec's Jacobian 1/(0/sz) is inf.
        out.append((f"{curve}_d3_p1_op6_gauss300", curve, 3, 8, 1, 6, ("gauss", 300)))
        out.append((f"{curve}_d3_p1_op6_ex1L4", curve, 3, 6, 1, 6, ("ex1", 4)))
        # HeatMat<3>::cgSolve (unpreconditioned CG, relative L-infinity stop);
        # the driver's op 7, stored as op 1 (its matVec outputs are HeatMat's)
        out.append((f"{curve}_d3_p1_op1_cg_gauss300", curve, 3, 8, 1, 7, ("gauss", 300)))
    # ot::DA<dim>::DA(func, ...): function2Octree of the two test fields of the
    # driver (1 / (eps + |x - c|^2)), then 2:1 balance
    for dim, md, order, tol in ((2, 8, 1, 0.2), (3, 7, 1, 1.0), (3, 7, 2, 1.0), (4, 6, 1, 4.0)):
        out.append((f"morton_d{dim}_p{order}_op2_f2o", "morton", dim, md, order, 2, ("f2o", tol)))
    for dim, md, order, tol in ((3, 7, 1, 1.0), (4, 6, 1, 4.0)):
        out.append((f"hilbert_d{dim}_p{order}_op2_f2o", "hilbert", dim, md, order, 2, ("f2o", tol)))
    return out


def vtu_arrays_ascii(path):
    """The data arrays of an ASCII VTU file (the reference's oct2vtu built
    with DENDRO_VTU_ASCII), by name."""
    import xml.etree.ElementTree as ET
    types = {"UInt32": np.uint32, "UInt64": np.uint64, "UInt8": np.uint8}
    return {da.get("Name"): np.array(da.text.split(), dtype=types[da.get("type")])
            for da in ET.parse(path).getroot().iter("DataArray")}


def vtu_goldens():
    """io::vtk::oct2vtu (the driver's op 8) of the Gaussian 300-point 3D tree
    in both curve orders: the tree as written, and the file's arrays."""
    os.makedirs(os.path.join(HERE, "vtu"), exist_ok=True)
    pts = trees.gaussian_points(300, 3, 8, seed=0)
    for curve in ("morton", "hilbert"):
        r = run_ref(curve, 3, 8, 1, 8, pts, None, 0, seed=1)
        a = vtu_arrays_ascii(os.path.join("/tmp", "dkt_golden_out.bin_vtu_0_1.vtu"))
        np.savez_compressed(os.path.join(HERE, "vtu", f"{curve}_d3_gauss300.npz"), curve=curve, dim=3, md=8,
                            tree_coords=r["tree_coords"], tree_levels=r["tree_levels"], **a)
        print("vtu", curve, r["tree_levels"].size, sorted(a))


def main(only=()):
    build_ref()
    if not only or "vtu" in only:
        vtu_goldens()
    for name, curve, dim, md, order, op, (src, arg) in cases():
        if only and not any(o in name for o in only):
            continue
        if src == "f2o":
            empty = np.zeros((0, dim), np.uint32)
            r = run_ref(curve, dim, md, order, op, empty, np.zeros(0, np.uint8), 3, seed=1, interp_tol=arg)
            inputs = dict(in_kind=3, in_coords=empty, in_levels=np.zeros(0, np.uint8), interp_tol=arg)
        elif src.startswith("gauss"):
            gmd = md - 1 if src == "gauss_shift" else md
            pts = trees.gaussian_points(arg, dim, gmd, seed=0)
            if src == "gauss_shift":
                # Same mesh one level finer in coordinates, so that Q2 node
                # spacing never collapses at the deepest level.
                tc, tl = None, None
                r0 = run_ref(curve, dim, gmd, 1, 0, pts, None, 0, seed=1)
                tc, tl = r0["tree_coords"] << np.uint32(1), r0["tree_levels"]
                r = run_ref(curve, dim, md, order, op, tc, tl, 1, seed=1)
                inputs = dict(in_kind=1, in_coords=tc, in_levels=tl)
            else:
                r = run_ref(curve, dim, md, order, op, pts, None, 0, seed=1)
                inputs = dict(in_kind=0, in_coords=pts, in_levels=np.zeros(0, np.uint8))
        else:
            gen = getattr(trees, "example" + src[-1])
            c, lv = gen(dim, arg, md)
            r = run_ref(curve, dim, md, order, op, c, lv, 2, seed=1)
            inputs = dict(in_kind=2, in_coords=c, in_levels=lv)
        extra = {}
        if op == 7:
            extra = dict(cg_tol=CG_TOL, cg_max_iter=CG_MAX_ITER, cg_status=r["cg_status"],
                         cg_resid=r["cg_resid"], cg_iters=r["cg_iters"], cg_b=r["cg_b"], cg_x=r["cg_x"])
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"), **extra,
            curve=curve, dim=dim, md=md, order=order, op=1 if op == 7 else op, seed=1, **inputs,
            tree_coords=r["tree_coords"], tree_levels=r["tree_levels"],
            node_coords=r["node_coords"], node_levels=r["node_levels"], bdry=r["bdry"],
            x=r["x"], y=r["y"], y_raw=r["y_raw"],
            ip0=r["ip0"], ip1=r["ip1"], Q1d=r["Q1d"], Dg=r["Dg"], W=r["W"])
        print(name, r["tree_levels"].size, r["node_levels"].size)


if __name__ == "__main__":
    main(sys.argv[1:])
