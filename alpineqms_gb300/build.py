"""Build libqms_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel; ``qms_exact.cu`` (the kernels
that must match the reference bit for bit) is compiled with ``-fmad=false``.
Output: ``alpineqms_gb300/_build/libqms_gb300.so``.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(BUILD, "libqms_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = {
    "qms_exact.cu": ["-fmad=false"],
    "qms_operator.cu": [],
    "qms_solver.cu": [],
    "qms_mg.cu": [],
    "qms_noalloc.cu": [],
    "qms_capi.cu": [],
    "qms_server.cpp": [],
    "qms_pl.cu": [],
}


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqms_gb300")


def _inputs_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for fn in sorted(os.listdir(d)):
            if fn.endswith((".cu", ".cuh", ".h", ".cpp")):
                with open(os.path.join(d, fn), "rb") as f:
                    h.update(fn.encode() + f.read())
    h.update(repr(SOURCES).encode() + repr(ARCH).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra_flags=None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    digest = _inputs_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp) and open(stamp).read() == digest:
        return LIB
    cc = nvcc()
    base = [cc, "-std=c++17", "-O3", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-I", INCLUDE, "-I", CSRC,
            *(extra_flags or [])]

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
        cmd = base + SOURCES[src] + ["-c", os.path.join(CSRC, src), "-o", obj]
        if verbose:
            print(" ".join(cmd))
        p = subprocess.run(cmd, capture_output=True, text=True)
        if p.returncode != 0:
            raise RuntimeError(f"nvcc failed on {src}:\n{p.stderr}")
        if verbose and p.stderr:
            print(p.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(compile_one, SOURCES))
    tmp = LIB + f".tmp{os.getpid()}"
    cmd = [cc, "-shared", *ARCH, "-o", tmp, *objs, "-lcudart"]
    p = subprocess.run(cmd, capture_output=True, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stderr}")
    os.replace(tmp, LIB)
    with open(stamp, "w") as f:
        f.write(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
