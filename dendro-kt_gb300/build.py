"""Build of the native library libdkt_gb300.so (in-tree, dendro-kt_gb300/_build/).

Every CUDA translation unit is compiled for sm_103a only
(-gencode arch=compute_103a,code=sm_103a), in parallel, then linked with the
host C++ unit into one shared library that exports the C ABI declared in
include/dkt_gb300.h and include/dkt_gb300_mesh.h.
"""
import concurrent.futures as cf
import fcntl
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libdkt_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU = ["dkt_da.cu", "dkt_plan.cu", "dkt_matvec.cu", "dkt_cg.cu", "dkt_capi.cu", "dkt_probe.cu", "dkt_q1fx.cu", "dkt_stale.cu", "dkt_tree.cu", "dkt_solve.cu", "dkt_tile.cu", "dkt_batch.cu", "dkt_serve.cu", "dkt_q2sf.cu"]
CPP = ["dkt_host.cpp"]


def nvcc():
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in CU + CPP]


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(REPO, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return hs


def up_to_date():
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(f) <= t for f in _sources() + _headers() + [__file__])


def _compile(src, verbose_ptxas=False):
    obj = os.path.join(OUT, os.path.basename(src) + ".o")
    if src.endswith(".cu"):
        # per-thread default streams: the work a host thread issues on stream 0
        # does not serialise with other threads' (concurrent served requests)
        cmd = [nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "--default-stream", "per-thread", "-Xcompiler",
               "-fPIC", "-c", src, "-o", obj]
        if verbose_ptxas:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-fPIC", "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile failed: %s\n%s\n%s" % (" ".join(cmd), r.stdout, r.stderr))
    return obj, r.stderr


def build(force=False, verbose_ptxas=False):
    if not force and up_to_date():
        return LIB
    os.makedirs(OUT, exist_ok=True)
    # one build at a time across processes (pool workers that all find the
    # library out of date): the others wait, then see it up to date
    with open(os.path.join(OUT, ".build.lock"), "w") as lock:
        fcntl.flock(lock, fcntl.LOCK_EX)
        if not force and up_to_date():
            return LIB
        return _build_locked(verbose_ptxas)


def _build_locked(verbose_ptxas):
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        res = list(ex.map(lambda s: _compile(s, verbose_ptxas), _sources()))
    objs = [o for o, _ in res]
    if verbose_ptxas:
        for _, err in res:
            print(err)
    tmp = "%s.%d.tmp" % (LIB, os.getpid())
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed: %s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force=True, verbose_ptxas="-v" in sys.argv))
