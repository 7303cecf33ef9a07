"""The reference-side binding of INTEGRATION.md, compiled and run.

oracle/build_binding.py takes INTEGRATION.md's `GPUPathTracingIntegrator` header and its
`Integrator::LoadIntegrator` branch verbatim, compiles them against the reference's own headers
(src/Integrators/Integrator.h:8-18, Integrator.cpp:14-47), links them with the reference's objects
and libc2g.so, and drives the reference's front end the way RayTracer does
(src/Core/RayTracer.cpp:11-43).  The CPU tests check that it builds, that the factory still builds
the reference's own integrators, and that a failure inside the library reaches the reference as an
exception; the GPU test renders the Cornell box at its full configuration through the reference's
`Integrator::Render` into its `FrameBuffer` and compares the image with c2g_film_image's.
"""
import ctypes as C
import json
import os

import numpy as np
import pytest

from crystal2_gb300 import scenes


@pytest.fixture(scope="module")
def bind_lib():
    from oracle import build_binding
    try:
        path = build_binding.build()
    except FileNotFoundError as e:  # no reference tree and no scratch copy on this host
        pytest.skip(f"reference sources unavailable: {e}")
    lib = C.CDLL(path)
    lib.bind_render.argtypes = [C.c_char_p, C.c_char_p, C.c_void_p, C.c_int, C.POINTER(C.c_int), C.POINTER(C.c_int),
                                C.c_char_p, C.c_int]
    lib.bind_render.restype = C.c_int
    return lib


def _render(lib, cp, sp, w, h):
    out = np.zeros(w * h * 3, np.float32)
    W, H = C.c_int(0), C.c_int(0)
    err = C.create_string_buffer(1024)
    rc = lib.bind_render(cp.encode(), sp.encode(), out.ctypes.data, out.size, C.byref(W), C.byref(H), err, 1024)
    return rc, out.reshape(h, w, 3), err.value.decode()


def _set_type(cp, integrator):
    cfg = json.load(open(cp))
    cfg["Integrator"]["Type"] = integrator
    json.dump(cfg, open(cp, "w"))


def test_binding_registers_in_the_reference_factory(bind_lib):
    from oracle import build_binding
    header, branch = build_binding.binding_sources()
    factory = build_binding.patched_factory(branch)
    assert 'type == "GPUPathTracer"' in factory and factory.index('"DirectLight"') < factory.index('"GPUPathTracer"')
    assert "class GPUPathTracingIntegrator : public Integrator" in header
    assert hasattr(bind_lib, "bind_render")


def test_reference_integrators_still_load_beside_the_binding(bind_lib, tmp_path):
    """The reference's own PathTracer branch of the patched factory renders on the CPU."""
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=16, height=16, spp=2, threads=2)
    rc, img, err = _render(bind_lib, cp, sp, 16, 16)
    assert rc == 0, err
    assert np.isfinite(img).all() and img.mean() > 0


def _missing_obj_scene(tmp_path):
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=16, height=16, spp=2, threads=2)
    _set_type(cp, "GPUPathTracer")
    scn = json.load(open(sp))
    scn["Scene"]["Objects"][0]["Shape"]["ObjFile"] = str(tmp_path / "missing.obj")
    bad = str(tmp_path / "bad_scene.json")
    json.dump(scn, open(bad, "w"))
    return cp, bad


def test_binding_reports_library_errors_as_exceptions(bind_lib, tmp_path):
    """A failing c2g call surfaces in the reference as an exception carrying the library's message
    (the integrator's constructor throws).  Without a GPU the context cannot be created; with one,
    the library rejects a scene whose OBJ file is missing (the reference's loader only prints)."""
    torch = pytest.importorskip("torch")
    cp, bad = _missing_obj_scene(tmp_path)
    rc, _, err = _render(bind_lib, cp, bad, 16, 16)
    assert rc == 1
    if torch.cuda.is_available():
        assert "missing.obj" in err
    else:
        assert "no CUDA device" in err


@pytest.mark.gpu
def test_binding_renders_cornell_through_the_reference_framebuffer(bind_lib, tmp_path):
    from crystal2_gb300 import Context
    from crystal2_gb300 import _native as N
    cp, sp = scenes.cornell(str(tmp_path / "c"))  # 256 x 256, 64 spp, depth 8
    _set_type(cp, "GPUPathTracer")
    rc, img, err = _render(bind_lib, cp, sp, 256, 256)
    assert rc == 0, err
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    ctx.render(ctx.render_params())
    ref_img = ctx.image()
    np.testing.assert_allclose(img, ref_img, rtol=1e-6, atol=0)
    assert img.mean() > 0.05
