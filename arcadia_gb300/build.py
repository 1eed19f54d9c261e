"""Builds ``arcadia_gb300/libarc_trace.so`` for sm_103a (in-tree; objects in ``arcadia_gb300/_build``).

Traversal translation units are compiled with ``--fmad=false --prec-div=true --prec-sqrt=true`` (the
canonical arithmetic the bit-exact hits rely on); the host builder with ``-ffp-contract=off``.
Run as ``python -m arcadia_gb300.build``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libarc_trace.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CANONICAL = ["--fmad=false", "--prec-div=true", "--prec-sqrt=true", "--ftz=false"]
CU_UNITS = {
    "arc_kernels.cu": CANONICAL,
    "arc_capi.cu": CANONICAL,
    "arc_sharc.cu": CANONICAL,
    "arc_nrc.cu": [],
    "arc_noalloc.cu": CANONICAL,
    "arc_edit.cu": CANONICAL,
    "arc_restir.cu": CANONICAL,
}
CPP_UNITS = ["arc_world.cpp"]


def _nvcc() -> str:
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(p):
        raise RuntimeError("nvcc not found")
    return p


def _sources_newer(obj: str, deps: list[str]) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(d) > t for d in deps)


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    inc = os.path.join(HERE, "..", "include", "arc")
    hs += [os.path.join(inc, f) for f in os.listdir(inc)]
    return hs


def _compile(cmd: list[str]) -> tuple[int, str]:
    r = subprocess.run(cmd, capture_output=True, text=True)
    return r.returncode, " ".join(cmd) + "\n" + r.stdout + r.stderr


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    hdrs = _headers()
    jobs, objs = [], []
    for src, extra in CU_UNITS.items():
        path = os.path.join(CSRC, src)
        if not os.path.exists(path):
            continue
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [path] + hdrs):
            jobs.append([nvcc, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", *extra, "-c", path, "-o", obj])
    for src in CPP_UNITS:
        path = os.path.join(CSRC, src)
        obj = os.path.join(OUT_DIR, src + ".o")
        objs.append(obj)
        if force or _sources_newer(obj, [path] + hdrs):
            jobs.append(["g++", "-O3", "-std=c++17", "-fPIC", "-fopenmp", "-ffp-contract=off", "-fno-fast-math", "-Wall",
                         "-c", path, "-o", obj])
    with cf.ThreadPoolExecutor(max_workers=max(1, len(jobs))) as ex:
        for rc, log in ex.map(_compile, jobs):
            if verbose or rc:
                print(log, file=sys.stderr)
            if rc:
                raise RuntimeError("compile failed:\n" + log)
    if force or jobs or not os.path.exists(LIB):
        cmd = [nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-Xcompiler", "-fopenmp", "-lgomp"]
        rc, log = _compile(cmd)
        if verbose or rc:
            print(log, file=sys.stderr)
        if rc:
            raise RuntimeError("link failed:\n" + log)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
