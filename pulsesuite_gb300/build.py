"""Build libsbe_gb300.so in-tree with nvcc for sm_103a (GB300).

Each .cu file under csrc/ is compiled in parallel to an object in _build/, then
linked into pulsesuite_gb300/libsbe_gb300.so.  Objects are rebuilt only when a
source or header is newer.  Usage: ``python -m pulsesuite_gb300.build``.
"""

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsbe_gb300.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC]
# per-file extra flags: the table builder must round like the reference's NumPy
# expressions (no fused multiply-add contraction).
EXTRA = {"sbe_tables.cu": ["-fmad=false"]}


def nvcc():
    exe = shutil.which("nvcc")
    if exe:
        return exe
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libsbe_gb300")


def _newest_header():
    t = 0.0
    for d in (CSRC, INCLUDE):
        for f in os.listdir(d):
            if f.endswith((".cuh", ".h")):
                t = max(t, os.path.getmtime(os.path.join(d, f)))
    return t


def _compile(src, obj, hdr_time, verbose):
    if os.path.exists(obj):
        ot = os.path.getmtime(obj)
        if ot >= os.path.getmtime(src) and ot >= hdr_time:
            return obj, ""
    cmd = [nvcc(), "-c", src, "-o", obj] + ARCH + COMMON + EXTRA.get(os.path.basename(src), [])
    if verbose:
        cmd.insert(1, "-Xptxas=-v")
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{p.stdout}\n{p.stderr}")
    return obj, p.stderr


def build(verbose=False, jobs=None):
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))
    hdr = _newest_header()
    objs = []
    logs = []
    with cf.ThreadPoolExecutor(max_workers=jobs or min(8, os.cpu_count() or 4)) as ex:
        futs = [ex.submit(_compile, s, os.path.join(BUILD, os.path.basename(s) + ".o"), hdr, verbose)
                for s in srcs]
        for f in futs:
            o, log = f.result()
            objs.append(o)
            if log:
                logs.append(log)
    need_link = not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB)
                                                for o in objs)
    if need_link:
        tmp = LIB + ".tmp"
        cmd = [nvcc(), "-shared", "-o", tmp] + objs + ARCH + ["-Xcompiler", "-fPIC"]
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"link failed:\n{p.stdout}\n{p.stderr}")
        os.replace(tmp, LIB)
    if verbose:
        for log in logs:
            sys.stderr.write(log)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
