"""Builds libmrg.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit under csrc/ is compiled by nvcc in parallel and linked
into mri_recon_gb300/_lib/libmrg.so.  Objects are rebuilt only when a source
or header is newer than the object.
"""
import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
SRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libmrg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _flags(verbose_ptxas=False):
    f = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC,-ffp-contract=off",
                "-I", os.path.join(ROOT, "include"), "-I", SRC]
    if verbose_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src, obj, verbose_ptxas):
    cmd = [nvcc()] + _flags(verbose_ptxas) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return r.stderr


def build(force=False, verbose_ptxas=False, jobs=None):
    os.makedirs(OUT, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(SRC, "*.cu")) + glob.glob(os.path.join(SRC, "*.cpp")))
    headers = (glob.glob(os.path.join(SRC, "*.h")) + glob.glob(os.path.join(SRC, "*.cuh")) +
               glob.glob(os.path.join(ROOT, "include", "*.h")))
    hdr_t = max(os.path.getmtime(h) for h in headers)
    todo, objs = [], []
    for s in srcs:
        o = os.path.join(OUT, os.path.basename(s) + ".o")
        objs.append(o)
        if force or verbose_ptxas or not os.path.exists(o) or os.path.getmtime(o) < max(os.path.getmtime(s), hdr_t):
            todo.append((s, o))
    logs = {}
    if todo:
        with cf.ThreadPoolExecutor(max_workers=jobs or min(len(todo), os.cpu_count() or 4)) as ex:
            futs = {ex.submit(_compile, s, o, verbose_ptxas): s for s, o in todo}
            for f in cf.as_completed(futs):
                logs[futs[f]] = f.result()
    if todo or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart_static", "-lrt", "-lpthread", "-ldl"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    return logs


if __name__ == "__main__":
    logs = build(force="--force" in sys.argv, verbose_ptxas="-v" in sys.argv)
    for k, v in logs.items():
        if v.strip():
            print("==", os.path.basename(k))
            print(v)
    print(LIB)
