"""Binary I/O for the reference oracle driver (oracle/ref/ref_driver.cpp).

Test infrastructure: writes driver inputs and parses its outputs.  Used only by
the fixture generator in this folder, which runs in a container that has the
reference sources.
"""
import struct
import numpy as np


def write_input(path, dim, max_depth, order, op, coords, levels=None, input_kind=0,
                n_calls=1, seed=1, x=None, interp_tol=None, cg_tol=None, cg_max_iter=None):
    coords = np.ascontiguousarray(coords, dtype=np.uint32).reshape(-1, dim)
    with open(path, "wb") as f:
        f.write(b"DKTI")
        f.write(struct.pack("<6i", dim, max_depth, order, op, input_kind, n_calls))
        f.write(struct.pack("<Q", seed))
        f.write(struct.pack("<Q", coords.shape[0]))
        f.write(coords.tobytes())
        if input_kind != 0:
            f.write(np.ascontiguousarray(levels, dtype=np.uint8).tobytes())
        if x is None:
            f.write(struct.pack("<Q", 0))
        else:
            x = np.ascontiguousarray(x, dtype=np.float64)
            f.write(struct.pack("<Q", x.size))
            f.write(x.tobytes())
        if input_kind == 3:
            f.write(struct.pack("<d", interp_tol))
        if op == 7:
            f.write(struct.pack("<di", cg_tol, cg_max_iter))


def read_output(path, dim):
    buf = open(path, "rb").read()
    off = 0

    def take(dtype, n):
        nonlocal off
        a = np.frombuffer(buf, dtype=dtype, count=n, offset=off)
        off += a.nbytes
        return a.copy()

    assert buf[:4] == b"DKTO"
    off = 4
    out = {}
    n = int(take(np.uint64, 1)[0])
    out["tree_coords"] = take(np.uint32, n * dim).reshape(n, dim)
    out["tree_levels"] = take(np.uint8, n)
    n = int(take(np.uint64, 1)[0])
    out["node_coords"] = take(np.uint32, n * dim).reshape(n, dim)
    out["node_levels"] = take(np.uint8, n)
    n = int(take(np.uint64, 1)[0])
    out["bdry"] = take(np.uint32, n)
    n = int(take(np.uint64, 1)[0])
    out["x"] = take(np.float64, n)
    n = int(take(np.uint64, 1)[0])
    out["y"] = take(np.float64, n)
    n = int(take(np.uint64, 1)[0])
    out["y_raw"] = take(np.float64, n)
    out["t_tree"], out["t_da"], out["t_matvec"] = take(np.float64, 3)
    m = int(take(np.int32, 1)[0])
    out["ip0"] = take(np.float64, m * m).reshape(m, m)
    out["ip1"] = take(np.float64, m * m).reshape(m, m)
    out["Q1d"] = take(np.float64, m * m).reshape(m, m)
    out["Dg"] = take(np.float64, m * m).reshape(m, m)
    out["W"] = take(np.float64, m)
    if off < len(buf):
        # op 7: HeatMat::cgSolve status, final relative L-infinity residual,
        # iterations, right-hand side and solution
        out["cg_status"] = int(take(np.int32, 1)[0])
        out["cg_resid"] = float(take(np.float64, 1)[0])
        out["cg_iters"] = int(take(np.int32, 1)[0])
        n = int(take(np.uint64, 1)[0])
        out["cg_b"] = take(np.float64, n)
        n = int(take(np.uint64, 1)[0])
        out["cg_x"] = take(np.float64, n)
    return out
