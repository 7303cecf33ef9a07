"""The allocation-free render entry point (c2g_render_noalloc).

It serves callers that cannot call cudaMalloc while they render: applications that own all
device memory through their own pool and give plug-ins no allocation rights, or frame loops that
cannot afford cudaMalloc's implicit synchronisation.  Its working memory is a fixed-size array
inside the library, so it must produce exactly what the allocating entry point (c2g_render)
produces, call after call, even though every call reuses the same array.  That holds for both
integrators it accepts: the path tracer, and direct lighting, whose paths keep walking through
surfaces without a material past the configured depth.
"""
import json

import numpy as np
import pytest

from crystal2_gb300 import Context, scenes
from crystal2_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from crystal2_gb300 import build
    build.build()


def _reference_film(cp, sp):
    ctx = Context(0)
    ctx.load(cp, sp)
    ctx.render(ctx.render_params())
    s, w = ctx.film()
    return ctx, s, w


def _noalloc(ctx, torch, params):
    film = torch.zeros((params.height, params.width, 4), dtype=torch.float32, device="cuda")
    torch.cuda.synchronize()
    import ctypes as C
    ctx.check(ctx._lib.c2g_render_noalloc(ctx.handle, C.byref(params), film.data_ptr(), None))
    out = film.cpu().numpy()
    return out[..., :3], out[..., 3]


def _with_integrator(cp, integrator, depth):
    cfg = json.load(open(cp))
    cfg["Integrator"]["Type"] = integrator
    cfg["Integrator"]["Depth"] = depth
    json.dump(cfg, open(cp, "w"))


@pytest.mark.parametrize("scene,integrator,depth", [
    ("cornell", "PathTracer", 8),
    ("material_box", "PathTracer", 8),
    ("material_box", "DirectLight", 1),
    ("material_box", "DirectLight", 8),
])
def test_noalloc_render_matches_render_twice(scene, integrator, depth, tmp_path):
    torch = pytest.importorskip("torch")
    if scene == "cornell":
        cp, sp = scenes.cornell(str(tmp_path / scene), width=48, height=40, spp=8)
    else:
        cp, sp = scenes.material_box(str(tmp_path / scene), width=40, height=32, spp=4)
    _with_integrator(cp, integrator, depth)
    ctx, s_ref, w_ref = _reference_film(cp, sp)
    p = ctx.render_params()
    for _ in range(2):  # the second call reuses the scratch the first one left behind
        s, w = _noalloc(ctx, torch, p)
        assert np.array_equal(w, w_ref)
        np.testing.assert_allclose(s, s_ref, rtol=1e-6, atol=1e-7)
    if integrator == "DirectLight":
        # material_box's panel and emitter quad have no material: direct lighting sees through
        # them, and the frame is lit (the comparison above is not between two black films)
        assert (s.max(-1) > 0).mean() >= 0.5


def test_noalloc_rejects_frames_beyond_its_limit(tmp_path):
    torch = pytest.importorskip("torch")
    cp, sp = scenes.cornell(str(tmp_path / "big"), width=256, height=256, spp=1)
    ctx = Context(0)
    ctx.load(cp, sp)
    with pytest.raises(N.C2GError) as e:
        _noalloc(ctx, torch, ctx.render_params())
    assert e.value.code == N.C2G_ERR_INVALID
    assert "exceeds the maximum" in str(e.value)
