"""The allocation-free feMatrix::matVec entry point.

dkt_fematrix_matvec_noalloc serves callers that cannot allocate device memory
while a product runs (a loop that reserved its device-memory budget up front,
or code that must not let cudaMalloc/cudaFree stall the device).  Its scratch
lives in a fixed device array; these tests call it through the C ABI and
check it against the regular entry point on two calls in a row (on meshes
with and without static-parent-buffer reads), that a call allocates no device
memory (the device's stream-ordered pool, its free memory and torch's
allocator are unchanged across it), and that it refuses plans larger than its
scratch.  This file is collected last."""
import ctypes

import numpy as np
import pytest

import __graft_entry__ as ge
import trees

pytestmark = pytest.mark.gpu
TOL = 1e-12


@pytest.fixture(scope="module")
def dkt():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return ge.load_package()


def _rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


class _DeviceMemory:
    """Device-memory counters through the driver API: the default
    stream-ordered pool's bytes in use and their high-water mark (reset
    before a call, so an allocation freed again within the call still shows),
    and the device's free memory."""

    USED_CURRENT, USED_HIGH = 7, 8     # CU_MEMPOOL_ATTR_USED_MEM_CURRENT / _HIGH

    def __init__(self):
        self.cu = ctypes.CDLL("libcuda.so.1")
        dev = ctypes.c_int(0)
        assert self.cu.cuCtxGetDevice(ctypes.byref(dev)) == 0
        self.pool = ctypes.c_void_p()
        assert self.cu.cuDeviceGetDefaultMemPool(ctypes.byref(self.pool), dev) == 0

    def _attr(self, a):
        v = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolGetAttribute(self.pool, a, ctypes.byref(v)) == 0
        return v.value

    def reset_high(self):
        z = ctypes.c_uint64(0)
        assert self.cu.cuMemPoolSetAttribute(self.pool, self.USED_HIGH, ctypes.byref(z)) == 0

    def snapshot(self):
        free, total = ctypes.c_size_t(0), ctypes.c_size_t(0)
        assert self.cu.cuMemGetInfo_v2(ctypes.byref(free), ctypes.byref(total)) == 0
        return self._attr(self.USED_CURRENT), self._attr(self.USED_HIGH), free.value


def _moving_ball_level5(dkt):
    tc, tl = dkt.moving_ball_tree(max_depth=10, level=5, radius=0.2, halfwidth=2.0 ** -5, device=True)
    return dkt.DA(tc, tl, 4, order=1, max_depth=10)


@pytest.mark.parametrize("dim,order,op", [(3, 1, 2), (4, 1, 2), (3, 2, 2), (2, 1, 0), (4, 1, "ball")])
def test_noalloc_matches_regular_entry_point_twice(dkt, dim, order, op):
    """Two calls in a row against dkt_fematrix_matvec; "ball": the 4D
    moving-ball mesh at level 5, whose products read 4,680 stale slots of the
    reference's static parent buffer."""
    import torch
    md = 9
    ball = op == "ball"
    if ball:
        da, op = _moving_ball_level5(dkt), dkt.OP_LAPMASS
    else:
        pts = dkt.gaussian_points(1500 if dim < 4 else 200, dim, md - 1, seed=11)
        tc, tl = dkt.tree_from_points(pts, dim, md - 1)
        tc = tc << np.uint32(1)
        da = dkt.DA(tc, tl, dim, order=order, max_depth=md)
    A = dkt.Matrix(da, op=op)
    if ball:
        assert A.stats()["stale_slots"] > 0
    L = dkt.load()
    for call, seed in enumerate((21, 22)):
        x = torch.from_numpy(dkt.uniform_pm1(seed, da.n)).cuda()
        y_ref = torch.empty_like(x)
        y_new = torch.full_like(x, float("nan"))
        A.matvec(x, y_ref)
        rc = L.dkt_fematrix_matvec_noalloc(A._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y_new.data_ptr()),
                                           1.0, None)
        assert rc == dkt.OK, L.dkt_last_error()
        torch.cuda.synchronize()
        a, b = y_new.cpu().numpy(), y_ref.cpu().numpy()
        assert np.all(np.isfinite(a))
        assert _rel(a, b) <= TOL, (call, _rel(a, b))


def test_noalloc_allocates_no_device_memory(dkt):
    """Across a call (after a first one, which loads its kernels), the
    default pool's bytes in use and their high-water mark, the device's free
    memory and torch's allocated bytes stay where they were."""
    import torch
    da = _moving_ball_level5(dkt)
    A = dkt.Matrix(da, op=dkt.OP_LAPMASS)
    L = dkt.load()
    x = torch.from_numpy(dkt.uniform_pm1(23, da.n)).cuda()
    y = torch.empty_like(x)
    args = (A._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 1.0, None)
    assert L.dkt_fematrix_matvec_noalloc(*args) == dkt.OK, L.dkt_last_error()
    torch.cuda.synchronize()
    mem = _DeviceMemory()
    mem.reset_high()
    used0, _, free0 = mem.snapshot()
    torch0 = torch.cuda.memory_allocated()
    assert L.dkt_fematrix_matvec_noalloc(*args) == dkt.OK, L.dkt_last_error()
    torch.cuda.synchronize()
    used1, high1, free1 = mem.snapshot()
    assert used1 == used0 and high1 <= used0, (used0, used1, high1)
    assert free1 == free0, (free0, free1)
    assert torch.cuda.memory_allocated() == torch0


def test_noalloc_rejects_plans_beyond_its_scratch(dkt):
    dim, md, L = 3, 8, 7      # 129^3 = 2,146,689 nodes > 1,048,576
    c, lv = trees.example2(dim, L, md)
    da = dkt.DA(c, lv, dim, order=1, max_depth=md, sorted_tree=False)
    A = dkt.Matrix(da, op=dkt.OP_LAPMASS)
    import torch
    x = torch.zeros(da.n, dtype=torch.float64, device="cuda")
    y = torch.empty_like(x)
    lib = dkt.load()
    rc = lib.dkt_fematrix_matvec_noalloc(A._h, ctypes.c_void_p(x.data_ptr()), ctypes.c_void_p(y.data_ptr()), 1.0, None)
    assert rc == dkt.E_ARG
    assert b"exceed" in lib.dkt_last_error()
