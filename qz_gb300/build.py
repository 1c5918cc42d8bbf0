"""Builds libqzgpu.so (the CUDA kernels + C ABI) in-tree for sm_103a.

Each translation unit is compiled by nvcc in parallel, then linked into
``qz_gb300/_lib/libqzgpu.so``.  Only one ``-gencode`` target (sm_103a) is built;
the same recipe runs on x86_64 and aarch64 hosts.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT, "libqzgpu.so")
# libbsc's BWT-stage symbols over the library (plain C object, linked by a
# caller together with libqzgpu.so in place of libbsc's own bwt object)
SHIM_SRC = os.path.join(CSRC, "bsc_bwt_shim.c")
SHIM_OBJ = os.path.join(OUT, "bsc_bwt_shim.o")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", "-I", os.path.join(ROOT, "include")]


def _nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libqzgpu")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _headers() -> list[str]:
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    inc = os.path.join(ROOT, "include")
    hs += [os.path.join(inc, f) for f in os.listdir(inc) if f.endswith(".h")]
    return sorted(hs)


def _stamp(extra: list[str]) -> str:
    h = hashlib.sha256()
    for p in sources() + _headers() + [SHIM_SRC]:
        with open(p, "rb") as f:
            h.update(p.encode() + f.read())
    h.update(" ".join(NVCC_FLAGS + ARCH + extra).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    extra = list(extra or [])
    os.makedirs(OUT, exist_ok=True)
    stamp_path = os.path.join(OUT, "stamp.txt")
    stamp = _stamp(extra)
    if not force and os.path.exists(LIB) and os.path.exists(SHIM_OBJ) and os.path.exists(stamp_path):
        with open(stamp_path) as f:
            if f.read().strip() == stamp:
                return LIB
    nvcc = _nvcc()
    objs = []
    cmds = []
    for src in sources():
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        objs.append(obj)
        cmds.append([nvcc, *ARCH, *NVCC_FLAGS, *extra, "-c", src, "-o", obj])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)

    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        raise RuntimeError("a C compiler (gcc) is required to build the libbsc shim object")
    cmds.append([cc, "-std=c99", "-O2", "-fPIC", "-Wall", "-Wextra", "-I", os.path.join(ROOT, "include"), "-c",
                 SHIM_SRC, "-o", SHIM_OBJ])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(cmds))) as ex:
        list(ex.map(run, cmds))
    tmp = LIB + ".tmp"
    run([nvcc, *ARCH, "-shared", "-o", tmp, *objs, "-lpthread"])
    os.replace(tmp, LIB)
    with open(stamp_path, "w") as f:
        f.write(stamp)
    return LIB


if __name__ == "__main__":
    verbose = "-v" in sys.argv
    extra = ["-Xptxas", "-v"] if "--ptxas" in sys.argv else []
    print(build(force=True, verbose=verbose or bool(extra), extra=extra))
