"""In-tree build of ``crystal2_gb300/libc2g.so`` (C++ host library + sm_103a CUDA kernels).

nvcc compiles the CUDA translation units for ``sm_103a`` only; g++ compiles the host sources with
``-ffp-contract=off`` (scene preprocessing must round like the reference) and the objects are
linked by nvcc into one shared library exposing the C ABI of ``include/c2g.h``.  Objects go to
``crystal2_gb300/_build/`` and every translation unit compiles in parallel.
"""
from __future__ import annotations

import hashlib
import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libc2g.so")

HOST_SOURCES = ["host/json.cpp", "host/scene.cpp", "host/bvh.cpp", "capi.cpp"]
CUDA_SOURCES = ["kernels/render.cu", "kernels/guide.cu"]

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Extra nvcc options (e.g. -D C2G_SHADOW_MIN_BLOCKS=12 to try another register budget); part of the
# sources digest, so a change rebuilds.
EXTRA_NVCC = os.environ.get("C2G_NVCC_EXTRA", "").split()


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    raise FileNotFoundError("nvcc not found")


def _cuda_home() -> str:
    return os.path.dirname(os.path.dirname(os.path.realpath(_nvcc())))


def _sources_digest() -> str:
    h = hashlib.sha256()
    for root, _d, files in os.walk(CSRC):
        for f in sorted(files):
            p = os.path.join(root, f)
            h.update(p.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    with open(os.path.join(ROOT, "include", "c2g.h"), "rb") as fh:
        h.update(fh.read())
    with open(__file__, "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(EXTRA_NVCC).encode())
    return h.hexdigest()


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile and link ``libc2g.so``; returns its path.  Skips work when sources are unchanged."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "stamp")
    digest = _sources_digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    nvcc = _nvcc()
    cuda_inc = os.path.join(_cuda_home(), "include")
    inc = [f"-I{CSRC}", f"-I{os.path.join(ROOT, 'include')}"]
    cxx = os.environ.get("CXX", "g++")

    def host(src: str) -> str:
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        cmd = [cxx, "-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-Wall", "-Wno-unused-function",
               f"-I{cuda_inc}", *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {src}:\n{r.stderr[-6000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    def cuda(src: str) -> str:
        obj = os.path.join(BUILD, src.replace("/", "_") + ".o")
        cmd = [nvcc, *ARCH, "-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
               "-Xptxas", "-v" if verbose else "-O3", *EXTRA_NVCC, *inc, "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stderr[-8000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=max(2, os.cpu_count() or 2)) as ex:
        futs = [ex.submit(host, s) for s in HOST_SOURCES] + [ex.submit(cuda, s) for s in CUDA_SOURCES]
        objs = [f.result() for f in futs]
    tmp = LIB + ".tmp"
    cmd = [nvcc, *ARCH, "-shared", "-Xcompiler", "-pthread", "-o", tmp, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    import sys
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
