"""Builds rchol_gb300/librchol_gb300.so in place (sm_103a only).

The library is plain nvcc / g++ output: CUDA sources with
``-gencode arch=compute_103a,code=sm_103a``, host C++ with g++, linked against
the METIS archive that ships with the CUDA toolkit.  Translation units are
compiled in parallel; unchanged objects are reused.
"""

from __future__ import annotations

import glob
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "librchol_gb300.so")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def metis_archive() -> str:
    cands = sorted(glob.glob(os.path.join(CUDA_HOME, "targets", "*", "lib", "libmetis_static.a")))
    cands += sorted(glob.glob(os.path.join(CUDA_HOME, "lib64", "libmetis_static.a")))
    if not cands:
        raise RuntimeError("libmetis_static.a not found under " + CUDA_HOME)
    return cands[0]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
    return r.stdout + r.stderr


def _stale(obj, deps):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(OBJ, exist_ok=True)
    nvcc = os.path.join(CUDA_HOME, "bin", "nvcc")
    inc = ["-I", os.path.join(ROOT, "include"), "-I", CSRC]
    headers = glob.glob(os.path.join(CSRC, "*.hpp")) + glob.glob(os.path.join(ROOT, "include", "*.h"))
    jobs = []
    checks = bool(os.environ.get("RCHOL_DEVICE_CHECKS"))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cu"))):
        obj = os.path.join(OBJ, os.path.basename(src) + (".chk.o" if checks else ".o"))
        cmd = [nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *inc, "-c", src, "-o", obj]
        if os.environ.get("RCHOL_DEVICE_CHECKS"):  # diagnostic build: device-side bounds checks
            cmd.insert(1, "-DRCHOL_DEVICE_CHECKS")
        if ptxas_info:
            cmd.insert(1, "-Xptxas=-v")
        jobs.append((obj, cmd, [src, *headers]))
    for src in sorted(glob.glob(os.path.join(CSRC, "*.cpp"))):
        obj = os.path.join(OBJ, os.path.basename(src) + ".o")
        cmd = ["g++", "-O2", "-fPIC", "-std=c++17", "-Wall", "-pthread", *inc,
               "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]
        jobs.append((obj, cmd, [src, *headers]))
    todo = [j for j in jobs if _stale(j[0], j[2]) or ptxas_info]
    logs = []
    with ThreadPoolExecutor(max_workers=max(1, min(8, os.cpu_count() or 1))) as ex:
        for out in ex.map(lambda j: _run(j[1]), todo):
            logs.append(out)
    objs = [j[0] for j in jobs]
    stamp_path = os.path.join(OBJ, "link.stamp")
    stamp = "\n".join(objs)
    old = open(stamp_path).read() if os.path.exists(stamp_path) else ""
    if todo or not os.path.exists(LIB) or old != stamp:
        _run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, metis_archive(), "-lpthread"])
        with open(stamp_path, "w") as f:
            f.write(stamp)
    log = "\n".join(l for l in logs if l.strip())
    if verbose and log:
        print(log, file=sys.stderr)
    return log


if __name__ == "__main__":
    print(build(verbose=True, ptxas_info="-v" in sys.argv) or "built " + LIB)
