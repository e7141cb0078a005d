"""Builds the engine's shared library in-tree with nvcc (sm_103a only).

Output: qsim_gb300/_build/libqsim_gb300.so.  Translation units compile in
parallel; objects are rebuilt only when a source or header is newer.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libqsim_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-Xcompiler", "-fPIC",
          "-I" + os.path.join(ROOT, "include"),
          "-I" + os.path.join(HERE, "csrc"),
          "-I" + os.path.join(HERE, "host")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required")


def _sources():
    cu = sorted(glob.glob(os.path.join(HERE, "csrc", "*.cu")))
    cc = sorted(glob.glob(os.path.join(HERE, "host", "*.cc")))
    return cu, cc


def _headers():
    hs = glob.glob(os.path.join(HERE, "csrc", "*.cuh"))
    hs += glob.glob(os.path.join(HERE, "csrc", "*.h"))
    hs += glob.glob(os.path.join(HERE, "host", "*.h"))
    hs += glob.glob(os.path.join(ROOT, "include", "*.h"))
    hs += glob.glob(os.path.join(ROOT, "include", "qsim_gb300", "*.h"))
    return hs


def _stale(obj: str, src: str, newest_header: float) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return t < os.path.getmtime(src) or t < newest_header


def _compile(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    return cmd, r.returncode, r.stdout + r.stderr


def _check_arch_stamp() -> None:
    """Objects built on another host architecture are discarded."""
    import platform
    stamp = os.path.join(BUILD, "ARCH")
    arch = platform.machine()
    old = open(stamp).read().strip() if os.path.exists(stamp) else None
    if old != arch:
        shutil.rmtree(BUILD, ignore_errors=True)
        os.makedirs(BUILD, exist_ok=True)
        with open(stamp, "w") as f:
            f.write(arch + "\n")


def build(verbose: bool = False, ptxas_info: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    _check_arch_stamp()
    cu, cc = _sources()
    hdr = _headers()
    newest = max([os.path.getmtime(h) for h in hdr] + [0.0])
    jobs, objs = [], []
    for src in cu + cc:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        objs.append(obj)
        if not _stale(obj, src, newest):
            continue
        cmd = [nvcc()] + ARCH + COMMON + ["-lineinfo"]
        if src.endswith(".cu"):
            cmd += ["-x", "cu"]
            if ptxas_info:
                cmd += ["-Xptxas", "-v"]
        else:
            cmd += ["-x", "c++", "-Xcompiler", "-fopenmp"]
        cmd += ["-c", src, "-o", obj]
        jobs.append(cmd)
    workers = max(1, min(len(jobs), os.cpu_count() or 4))
    failed = []
    if jobs:
        with cf.ThreadPoolExecutor(workers) as ex:
            for cmd, rc, out in ex.map(_compile, jobs):
                if verbose or rc != 0 or ptxas_info:
                    sys.stderr.write(" ".join(cmd[-3:]) + "\n" + out)
                if rc != 0:
                    failed.append(cmd[-3])
    if failed:
        raise RuntimeError("compilation failed: " + ", ".join(failed))
    if jobs or not os.path.exists(LIB):
        link = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + [
            "-Xcompiler", "-fopenmp", "-lcudart"]
        _, rc, out = _compile(link)
        if rc != 0:
            raise RuntimeError("link failed:\n" + out)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, ptxas_info="--ptxas" in sys.argv))
