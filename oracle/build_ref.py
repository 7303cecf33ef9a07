#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref``: the reference renderer compiled from its own sources.

TEST INFRASTRUCTURE ONLY.  What this script builds is the checker the parity tests and the
CPU baseline use; no product code links, loads or calls it.

Crystal2 is MSVC-flavoured C++17.  g++ 13 compiles its hot path after six mechanical,
behaviour-neutral edits, applied here to a scratch copy under ``oracle/_ref/src`` (never
committed; ``oracle/_ref`` is git-ignored):

1. ``virtual ~X() = 0 {}`` (a pure-specifier on a definition, an MSVC extension) becomes
   ``virtual ~X() {}``.
2. ``std::exception("msg")`` (an MSVC-only constructor) becomes ``std::runtime_error("msg")``.
3. The redundant ``SJson::`` qualification on two SJson.cpp definitions is dropped.
4. ``std::pow(10.0, ll)`` in the SJson number parser becomes ``pow`` (same double overload).
5. ``<cmath> <stdexcept> <cstring> <cassert> <atomic> <condition_variable>`` are force-included.
6. The harness translation unit defines ``STB_IMAGE_IMPLEMENTATION`` (the GL engine normally
   does, deps/TREngine/Core/Render/Texture2D.cpp:3).

Nothing else in the reference changes.  ``-ffp-contract=off`` keeps float arithmetic free of
FMA contraction on both x86-64 and aarch64, which is what x86-64 g++ emits by default.

Layout of the scratch copy (mirrors the reference tree):
  oracle/_ref/src/src/...                         reference ``src/``
  oracle/_ref/src/deps/TREngine/deps/{glm,SJson,stbi}
  oracle/_ref/src/deps/TREngine/Core/Utils/...

Outputs: ``oracle/_ref/libc2ref.so`` (the reference objects plus ``oracle/ref_harness.cpp``).

Usage: ``python oracle/build_ref.py [--src /path/to/reference]``.  Without a reference tree
but with a scratch copy already present (the copy travels with the repository snapshot), the
library is rebuilt from the copy, which lets an aarch64 host rebuild it.
"""
from __future__ import annotations

import argparse
import hashlib
import os
import re
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
SCRATCH = os.path.join(OUT, "src")
LIB = os.path.join(OUT, "libc2ref.so")
HARNESS = os.path.join(HERE, "ref_harness.cpp")
# The reference checkout: $C2_REFERENCE_SRC, else a sibling directory ``reference`` of the repository.
DEFAULT_REF = os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")


def reference_tree() -> str:
    return os.environ.get("C2_REFERENCE_SRC") or DEFAULT_REF

# Reference translation units on the path (everything in src/ except the GL app shell and demos).
EXCLUDE = {"src/CrystalEngine.cpp", "src/Demos/BRDFDemo.cpp"}
EXTRA_TUS = [
    "deps/TREngine/deps/SJson/SJson.cpp",
    "deps/TREngine/Core/Utils/Threads/FixedThreadPool.cpp",
]

CXXFLAGS = [
    "-std=c++17", "-O2", "-fPIC", "-pthread", "-w", "-ffp-contract=off",
    "-include", "cmath", "-include", "stdexcept", "-include", "cstring",
    "-include", "cassert", "-include", "atomic", "-include", "condition_variable",
]


def _copy_tree(ref: str) -> None:
    if os.path.isdir(SCRATCH):
        shutil.rmtree(SCRATCH)
    os.makedirs(SCRATCH)
    shutil.copytree(os.path.join(ref, "src"), os.path.join(SCRATCH, "src"))
    for sub in ("deps/TREngine/deps/glm", "deps/TREngine/deps/SJson", "deps/TREngine/deps/stbi",
                "deps/TREngine/Core/Utils"):
        shutil.copytree(os.path.join(ref, sub), os.path.join(SCRATCH, sub))
    for root, _dirs, files in os.walk(SCRATCH):
        for f in files:
            os.chmod(os.path.join(root, f), 0o644)
        os.chmod(root, 0o755)


_PURE_DTOR = re.compile(r"(virtual\s+~\w+\s*\(\s*\))\s*=\s*0\s*\{\s*\}")


def _patch_tree() -> int:
    n = 0
    for root, _dirs, files in os.walk(SCRATCH):
        if "/glm" in root:
            continue
        for f in files:
            if not f.endswith((".h", ".hpp", ".cpp")):
                continue
            p = os.path.join(root, f)
            with open(p, "rb") as fh:
                raw = fh.read()
            txt = raw.decode("utf-8", errors="surrogateescape")
            new = _PURE_DTOR.sub(r"\1 {}", txt)                              # patch 1
            new = new.replace("std::exception(", "std::runtime_error(")      # patch 2
            new = new.replace("public std::exception", "public std::runtime_error")
            if f == "SJson.cpp":
                new = new.replace("std::string SJson::SJsonGetNodeTypeName", "std::string SJsonGetNodeTypeName")  # patch 3
                new = new.replace("std::shared_ptr<SJsonNode> SJson::SJsonParse", "std::shared_ptr<SJsonNode> SJsonParse")
                new = new.replace("std::pow(10.0,", "pow(10.0,")            # patch 4
            if new != txt:
                n += 1
                with open(p, "wb") as fh:
                    fh.write(new.encode("utf-8", errors="surrogateescape"))
    return n


def _sources() -> list[str]:
    tus = []
    for root, _dirs, files in os.walk(os.path.join(SCRATCH, "src")):
        for f in files:
            if f.endswith(".cpp"):
                rel = os.path.relpath(os.path.join(root, f), SCRATCH)
                if rel not in EXCLUDE:
                    tus.append(rel)
    tus += EXTRA_TUS
    return sorted(tus)


def _includes() -> list[str]:
    return ["-I" + os.path.join(SCRATCH, p) for p in
            ("src", "deps/TREngine/deps", "deps/TREngine", "deps")]


def build(ref: str | None = None, force: bool = False, jobs: int | None = None) -> str:
    """Build ``oracle/_ref/libc2ref.so``; return its path.  Raises on a failed compile."""
    if ref is None:
        ref = reference_tree()
    have_ref = os.path.isdir(os.path.join(ref, "src"))
    if have_ref and (force or not os.path.isdir(SCRATCH)):
        _copy_tree(ref)
        _patch_tree()
    if not os.path.isdir(SCRATCH):
        raise FileNotFoundError("no reference tree and no scratch copy under oracle/_ref/src")
    stamp = os.path.join(OUT, "harness.sha256")
    with open(HARNESS, "rb") as fh:
        digest = hashlib.sha256(fh.read()).hexdigest()
    if os.path.exists(LIB) and not force and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    objdir = os.path.join(OUT, "obj")
    os.makedirs(objdir, exist_ok=True)
    inc = _includes()
    cxx = os.environ.get("CXX", "g++")

    def compile_one(rel: str) -> str:
        obj = os.path.join(objdir, rel.replace("/", "_") + ".o")
        cmd = [cxx, *CXXFLAGS, *inc, "-c", os.path.join(SCRATCH, rel), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {rel}\n{r.stderr[-4000:]}")
        return obj

    tus = _sources()
    with ThreadPoolExecutor(max_workers=jobs or os.cpu_count() or 4) as ex:
        objs = list(ex.map(compile_one, tus))
    hobj = os.path.join(objdir, "ref_harness.o")
    r = subprocess.run([cxx, *CXXFLAGS, *inc, "-c", HARNESS, "-o", hobj], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("harness compile failed\n" + r.stderr[-6000:])
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, "-shared", "-pthread", "-o", tmp, hobj, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--src", default=None)
    ap.add_argument("--force", action="store_true")
    a = ap.parse_args()
    print(build(a.src, force=a.force))
    return 0


if __name__ == "__main__":
    sys.exit(main())
