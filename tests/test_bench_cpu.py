"""The benchmark's reference arm on the CPU, alone and under a 2-rank
torchrun (gloo): rank 0 alone prints one JSON line with the contract's keys,
the other rank exits 0 without work (replicas only, no collective on the
data path)."""
import json
import os
import subprocess
import sys

import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
ARGS = ["--impl", "reference", "--level", "3", "--steps", "1", "--warmup", "1", "--cpu-seconds", "0.2",
        "--cpu-procs", "2"]


def _lines(out):
    return [json.loads(l) for l in out.splitlines() if l.startswith("{")]


def _check(line):
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling", "dtype",
              "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["impl"] == "reference" and line["value"] > 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] == 2
    assert line["e2e"]["h2d_bytes_per_step"] == 0
    # one product of the whole mesh is the step it times; the requested
    # counts are echoed, not claimed
    assert line["steps"] == 1 and line["warmup"] == 0
    assert line["requested_steps"] == 1 and line["requested_warmup"] == 1


def test_reference_arm_single_process():
    r = subprocess.run([sys.executable, "bench.py", *ARGS], cwd=REPO, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1
    _check(lines[0])


def test_reference_arm_two_ranks_gloo():
    pytest.importorskip("torch")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node", "2",
           "--master-addr", "127.0.0.1", "--master-port", "29517", "bench.py", "--gpus", "2", *ARGS]
    r = subprocess.run(cmd, cwd=REPO, capture_output=True, text=True, timeout=900)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = _lines(r.stdout)
    assert len(lines) == 1   # rank 0 only
    _check(lines[0])
    assert lines[0]["n_gpus"] == 2


def test_reference_arm_mesh_equals_library_mesh():
    """The reference arm builds its meshes with the oracle's restatement of
    the moving-ball refinement and 2:1 balance (no GB300 library in that
    process); it reproduces the library's host-built tree cell for cell, and
    its level-2 partitions hold the same cells inside their partition cell."""
    import numpy as np
    import __graft_entry__ as ge
    import oracle_port as orc
    dkt = ge.load_package()
    orc.set_curve(4, 10)
    oc, ol = orc.moving_ball_tree(4)
    hc, hl = dkt.moving_ball_tree(max_depth=10, level=4)
    a = sorted(map(tuple, np.concatenate([oc, ol[:, None]], 1).tolist()))
    b = sorted(map(tuple, np.concatenate([hc, hl[:, None]], 1).tolist()))
    assert a == b
    k = 5                                        # level-2 cell, Morton digits (0, 5)
    pc, pl = orc.moving_ball_tree(4, part_level=2, part_index=k)
    anc = np.array([((k >> d) & 1) << 8 for d in range(4)], np.uint32)
    ins = lambda c, l: np.all((c >= anc) & (c < anc + 256), axis=1) & (l >= 2)
    assert set(map(tuple, np.concatenate([pc, pl[:, None]], 1)[ins(pc, pl)].tolist())) == \
        set(map(tuple, np.concatenate([oc, ol[:, None]], 1)[ins(oc, ol)].tolist()))
