#!/usr/bin/env python3
"""Build recipe for ``oracle/_ref/bind/libc2bind.so``: the reference renderer with the GPU integrator
registered in its factory, exactly as INTEGRATION.md tells a maintainer to do it.

TEST INFRASTRUCTURE ONLY.  It proves the reference-side binding compiles and links against the
reference's own headers and objects and this repository's ``libc2g.so``:

1. the ``GPUPathTracingIntegrator`` header is taken verbatim from INTEGRATION.md's first C++
   block and written to ``oracle/_ref/bind/src/Integrators/GPUPathTracingIntegrator.h``;
2. ``Integrator::LoadIntegrator`` (``src/Integrators/Integrator.cpp:14-47``) is copied from the
   patched reference tree (``oracle/_ref/src``, made by ``oracle/build_ref.py``) and the
   registration branch from INTEGRATION.md's second C++ block is inserted after the
   ``DirectLight`` branch, with the header included;
3. that translation unit and ``oracle/bind_driver.cpp`` (the reference's front end driven like
   ``RayTracer``) are compiled with the reference's flags and linked with every other reference
   object of ``oracle/_ref/obj`` and with ``libc2g.so``.

Usage: ``python oracle/build_binding.py``; returns the library path.  Needs ``oracle/_ref`` built.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, ROOT)

from oracle import build_ref  # noqa: E402

OUT = os.path.join(build_ref.OUT, "bind")
LIB = os.path.join(OUT, "libc2bind.so")
DOC = os.path.join(ROOT, "INTEGRATION.md")
DRIVER = os.path.join(HERE, "bind_driver.cpp")


def cpp_blocks(md_path: str = DOC) -> list[str]:
    """The ```cpp fenced blocks of a markdown file, in order."""
    with open(md_path) as fh:
        text = fh.read()
    return re.findall(r"```cpp\n(.*?)```", text, flags=re.S)


def binding_sources() -> tuple[str, str]:
    """(integrator header, factory branch) as INTEGRATION.md gives them."""
    blocks = cpp_blocks()
    header = next(b for b in blocks if "class GPUPathTracingIntegrator" in b)
    branch = next(b for b in blocks if 'type == "GPUPathTracer"' in b)
    return header, branch


def patched_factory(branch: str) -> str:
    """Integrator.cpp of the reference with the GPU branch registered after "DirectLight"."""
    src = os.path.join(build_ref.SCRATCH, "src", "Integrators", "Integrator.cpp")
    with open(src, "rb") as fh:
        text = fh.read().decode("utf-8-sig")
    at = text.index('type == "DirectLight"')
    m = re.compile(r"\n\s*else\s*\n").search(text, at)  # the chain's final else
    if m is None:
        raise RuntimeError("cannot find the end of LoadIntegrator's branch chain")
    text = text[:m.start()] + "\n" + branch.rstrip() + text[m.start():]
    return '#include "GPUPathTracingIntegrator.h"\n' + text


def build(force: bool = False) -> str:
    build_ref.build()
    header, branch = binding_sources()
    os.makedirs(os.path.join(OUT, "src", "Integrators"), exist_ok=True)
    hpath = os.path.join(OUT, "src", "Integrators", "GPUPathTracingIntegrator.h")
    fpath = os.path.join(OUT, "Integrator_gpu.cpp")
    factory = patched_factory(branch)
    inputs = {hpath: header, fpath: factory}
    changed = force or not os.path.exists(LIB)
    for p, txt in inputs.items():
        old = open(p).read() if os.path.exists(p) else None
        if old != txt:
            with open(p, "w") as fh:
                fh.write(txt)
            changed = True
    from crystal2_gb300 import build as libbuild
    c2g = libbuild.build()
    if not changed and os.path.getmtime(LIB) >= max(os.path.getmtime(c2g), os.path.getmtime(DRIVER)):
        return LIB
    cxx = os.environ.get("CXX", "g++")
    # the header sits beside the reference's own Integrators/ headers, as it would in the tree
    inc = ["-I" + os.path.join(OUT, "src"), "-I" + os.path.join(OUT, "src", "Integrators"),
           "-I" + os.path.join(build_ref.SCRATCH, "src", "Integrators"), *build_ref._includes(),
           "-I" + os.path.join(ROOT, "include")]
    objs = []
    for src in (fpath, DRIVER):
        obj = os.path.join(OUT, os.path.basename(src) + ".o")
        r = subprocess.run([cxx, *build_ref.CXXFLAGS, *inc, "-c", src, "-o", obj], capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"compile failed: {src}\n{r.stderr[-6000:]}")
        objs.append(obj)
    objdir = os.path.join(build_ref.OUT, "obj")
    ref_objs = sorted(os.path.join(objdir, f) for f in os.listdir(objdir)
                      if f.endswith(".o") and f not in ("ref_harness.o", "src_Integrators_Integrator.cpp.o"))
    libdir = os.path.dirname(c2g)
    tmp = LIB + ".tmp"
    r = subprocess.run([cxx, "-shared", "-pthread", "-o", tmp, *objs, *ref_objs, c2g, f"-Wl,-rpath,{libdir}"],
                       capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed\n" + r.stderr[-4000:])
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv))
