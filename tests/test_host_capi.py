"""The C-ABI library without a GPU: symbols, host-only scene loading, tree builds, errors."""
import ctypes as C
import json
import os
import re

import numpy as np
import pytest

from crystal2_gb300 import Context, scenes
from crystal2_gb300 import _native as N

from golden_util import GOLDEN, SCENES, SAMPLER_CASES, read_rgbe, sampler_scene

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module", autouse=True)
def built_library():
    from crystal2_gb300 import build
    build.build()


def declared_symbols():
    names = set()
    inc = os.path.join(ROOT, "include")
    for f in os.listdir(inc):
        if f.endswith(".h"):
            with open(os.path.join(inc, f)) as fh:
                txt = fh.read()
            names |= set(re.findall(r"\b(c2g_[a-z0-9_]+)\s*\(", txt))
    return names


def test_library_exports_every_declared_symbol():
    lib = C.CDLL(N.LIB_PATH)
    names = declared_symbols()
    assert names, "no declarations found"
    for n in sorted(names):
        assert hasattr(lib, n), n
    # the Python binding covers the whole ABI
    assert names <= set(N.SIGNATURES), names - set(N.SIGNATURES)


@pytest.mark.parametrize("name", list(SCENES))
def test_host_tree_matches_reference_golden(name, tmp_path):
    cp, sp = SCENES[name](str(tmp_path / name))
    ctx = Context(device=-1)
    ctx.load(cp, sp, tree=N.TREE_REF_EQUAL_COUNT)
    z = np.load(os.path.join(GOLDEN, f"bvh_{name}.npz"))
    assert np.array_equal(ctx.bvh_order(), z["order"])
    b, a, ax = ctx.bvh_nodes()
    assert np.array_equal(b.view(np.uint32), z["bounds_bits"])
    assert np.array_equal(a, z["a"]) and np.array_equal(ax, z["axis"])


def test_sah_build_keeps_reference_order_available(tmp_path):
    cp, sp = SCENES["spheres"](str(tmp_path / "s"))
    ctx = Context(device=-1)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    z = np.load(os.path.join(GOLDEN, "bvh_spheres.npz"))
    assert np.array_equal(ctx.bvh_order(), z["order"])


def test_render_params_follow_config(tmp_path):
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=40, height=30, spp=7, depth=5, accel="Brute")
    ctx = Context(device=-1)
    ctx.load(cp, sp)
    p = ctx.render_params()
    assert (p.width, p.height, p.spp, p.max_depth, p.accel) == (40, 30, 7, 5, N.ACCEL_BRUTE)
    assert ctx.num_objects() == 14 and ctx.num_lights() == 2


def _expect(code, fn):
    with pytest.raises(N.C2GError) as e:
        fn()
    assert e.value.code == code, str(e.value)


def test_error_codes(tmp_path):
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=8, height=8, spp=1)
    ctx = Context(device=-1)
    _expect(N.C2G_ERR_IO, lambda: ctx.load(str(tmp_path / "missing.json"), sp))
    bad = tmp_path / "bad.json"
    bad.write_text('{"Width": 8, "Height": ')
    _expect(N.C2G_ERR_PARSE, lambda: ctx.load(str(bad), sp))
    cfg = json.load(open(cp))
    scn = json.load(open(sp))
    # unknown material type -> invalid (Material.cpp:123-125)
    s2 = json.loads(json.dumps(scn))
    s2["Scene"]["Objects"][0]["Material"] = {"Type": "Velvet"}
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(cfg), json.dumps(s2)))
    # a Kd texture name the scene does not define -> invalid (Scene.cpp:69-77)
    s3 = json.loads(json.dumps(scn))
    s3["Scene"]["Objects"][0]["Material"] = {"Type": "Diffuse", "Kd": "Test"}
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(cfg), json.dumps(s3)))
    # an image in a format the loader does not decode (and nobody registered) -> unsupported
    jpg = tmp_path / "photo.jpg"
    jpg.write_bytes(bytes([0xFF, 0xD8, 0xFF, 0xE0]) + bytes(60))
    s3["Scene"]["Textures"] = {"Test": {"Path": str(jpg)}}
    _expect(N.C2G_ERR_UNSUPPORTED, lambda: ctx.load_text(json.dumps(cfg), json.dumps(s3)))
    # the same file decoded by the caller loads (c2g_register_image)
    ctx.register_image(str(jpg), np.full((2, 3, 3), 128, np.uint8))
    ctx.load_text(json.dumps(cfg), json.dumps(s3))
    # textured Oren-Nayar is unimplemented in the reference too (Material.cpp:103-108)
    s3["Scene"]["Objects"][0]["Material"] = {"Type": "OrenNayar", "Kd": "Test", "Sigma": 0.3}
    _expect(N.C2G_ERR_UNSUPPORTED, lambda: ctx.load_text(json.dumps(cfg), json.dumps(s3)))
    # unknown integrator / accelerator -> invalid (Integrator.cpp:37-43, Accelerator.cpp:20-23)
    c2 = json.loads(json.dumps(cfg))
    c2["Integrator"]["Type"] = "Photon"
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(c2), json.dumps(scn)))
    c3 = json.loads(json.dumps(cfg))
    c3["Acceleration"] = "Octree"
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(c3), json.dumps(scn)))
    # non-triangular OBJ face -> parse error
    quad = tmp_path / "quad.obj"
    quad.write_text("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvn 0 0 1\nf 1//1 2//1 3//1 4//1\n")
    s4 = json.loads(json.dumps(scn))
    s4["Scene"]["Objects"][0]["Shape"]["ObjFile"] = str(quad)
    _expect(N.C2G_ERR_PARSE, lambda: ctx.load_text(json.dumps(cfg), json.dumps(s4)))
    # device work on a host-only context -> bad state
    ctx.load(cp, sp)
    _expect(N.C2G_ERR_STATE, lambda: ctx.render(ctx.render_params()))
    _expect(N.C2G_ERR_STATE, lambda: ctx.trace_rays(np.zeros((1, 3), np.float32), np.ones((1, 3), np.float32)))


def test_json_numbers_follow_reference_parser(tmp_path):
    """Floats are accumulated digit by digit like SJson; the BVH bounds of a mesh translated by such
    numbers still match the reference (covered by the goldens), and ints stay ints."""
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=8, height=8, spp=3)
    cfg = json.load(open(cp))
    cfg["Width"] = 8
    ctx = Context(device=-1)
    ctx.load_text(json.dumps(cfg), open(sp).read())
    assert ctx.render_params().spp == 3


def test_textured_scene_loads_on_host(tmp_path):
    """Textures, per-triangle uvs and the six skybox faces load without a device; a truncated PPM
    raster is a parse error."""
    cp, sp = scenes.textured_yard(str(tmp_path / "t"))
    ctx = Context(device=-1)
    ctx.load(cp, sp)
    assert ctx.num_objects() == 6 and ctx.num_lights() == 3  # two area-light triangles + the point light
    scn = json.load(open(sp))
    bad = tmp_path / "short.ppm"
    bad.write_bytes(b"P6\n4 4\n255\n" + bytes(10))
    scn["Scene"]["Textures"]["floor"]["Path"] = str(bad)
    _expect(N.C2G_ERR_PARSE, lambda: ctx.load_text(open(cp).read(), json.dumps(scn)))
    scn = json.load(open(sp))
    scn["Scene"]["Skybox"]["Path"] = str(tmp_path / "nowhere")
    _expect(N.C2G_ERR_IO, lambda: ctx.load_text(open(cp).read(), json.dumps(scn)))


def test_hdr_writer_matches_reference_writer(tmp_path):
    """c2g_write_hdr against the reference's stbi_write_hdr (RayTracer.cpp:40) on the same float
    images: identical dimensions and identical RGBE pixels after decoding (flat scanlines below
    width 8, run-length scanlines otherwise)."""
    from crystal2_gb300 import write_hdr
    z = np.load(os.path.join(GOLDEN, "hdr_writer.npz"))
    keys = [k[4:] for k in z.files if k.startswith("img_")]
    assert len(keys) == 4
    for key in keys:
        img = z["img_" + key]
        path = str(tmp_path / f"{key}.hdr")
        write_hdr(path, img)
        ours = open(path, "rb").read()
        ref = z["file_" + key].tobytes()
        assert ours.startswith(b"#?RADIANCE\n")
        a, b = read_rgbe(ours), read_rgbe(ref)
        assert a.shape == b.shape == img.shape[:2] + (4,)
        assert np.array_equal(a, b), key
    with pytest.raises(N.C2GError):
        write_hdr(str(tmp_path / "no_such_dir" / "x.hdr"), np.zeros((2, 2, 3), np.float32))


def test_sampler_types_follow_reference_factory(tmp_path):
    """Sampler::LoadSampler (Sampler.cpp:10-53): Halton, Default and Stratified load; Stratified
    needs a square sample count; any other name is invalid."""
    for name in SAMPLER_CASES:
        cp, sp = sampler_scene(str(tmp_path), name)
        Context(device=-1).load(cp, sp)
    cfg = json.load(open(cp))
    scn = open(sp).read()
    ctx = Context(device=-1)
    cfg["Integrator"]["Sampler"]["Type"] = "Stratified"
    cfg["SamplesPerPixel"] = 8
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(cfg), scn))
    cfg["SamplesPerPixel"] = 16
    ctx.load_text(json.dumps(cfg), scn)
    cfg["Integrator"]["Sampler"]["Type"] = "Sobol"
    _expect(N.C2G_ERR_INVALID, lambda: ctx.load_text(json.dumps(cfg), scn))


def test_scene_without_objects_is_rejected(tmp_path):
    """A scene with no geometry (none at all, or only a point light) is C2G_ERR_INVALID: the
    reference's BVH build dereferences the missing objects and crashes on it."""
    cfg = scenes.config_json(13, 7, 2, 4)
    for name, objs in (("empty", []), ("point_only", [scenes.point_light((0, 2, 0), (10, 10, 10))])):
        cp, sp = scenes.write_scene(str(tmp_path), cfg, scenes.camera((0, 0, -4), (0, 0, 0), 40), objs, name)
        _expect(N.C2G_ERR_INVALID, lambda: Context(device=-1).load(cp, sp))


def test_new_entry_points_reject_bad_arguments(tmp_path):
    """Null pointers and a context without a device give status codes, never a crash."""
    lib = N.load_library()
    img = np.zeros((2, 3, 3), np.float32)
    assert lib.c2g_write_hdr(None, 3, 2, N.fptr(img)) == N.C2G_ERR_INVALID
    assert lib.c2g_write_hdr(str(tmp_path / "x.hdr").encode(), 0, 2, N.fptr(img)) == N.C2G_ERR_INVALID
    assert lib.c2g_write_hdr(str(tmp_path / "x.hdr").encode(), 3, 2, None) == N.C2G_ERR_INVALID
    assert lib.c2g_film_write_hdr(None, b"x.hdr") == N.C2G_ERR_INVALID
    assert lib.c2g_sampler_values(None, 1, None, None, None, 0, 1, None) == N.C2G_ERR_INVALID
    ctx = Context(device=-1)
    # no scene loaded
    assert lib.c2g_film_write_hdr(ctx.handle, str(tmp_path / "y.hdr").encode()) == N.C2G_ERR_STATE
    px = np.zeros(1, np.int32)
    out = np.zeros(2, np.float32)
    assert lib.c2g_sampler_values(ctx.handle, 1, N.iptr(px), N.iptr(px), N.iptr(px), 0, 1, N.fptr(out)) == N.C2G_ERR_STATE
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=8, height=8, spp=1)
    ctx.load(cp, sp)
    # a host-only context has no device to draw samples on
    assert lib.c2g_sampler_values(ctx.handle, 1, N.iptr(px), N.iptr(px), N.iptr(px), 0, 1, N.fptr(out)) != N.C2G_OK
    assert lib.c2g_sampler_values(ctx.handle, 1, N.iptr(px), N.iptr(px), N.iptr(px), -1, 1, N.fptr(out)) == N.C2G_ERR_INVALID


def test_tuning_entry_points_reject_bad_arguments():
    """Traversal block, guide training batch and batch configuration calls validate their
    arguments before touching a device: a null handle or an out-of-range value is an error code."""
    lib = N.load_library()
    assert lib.c2g_set_trace_block(None, 128) == N.C2G_ERR_INVALID
    assert lib.c2g_guide_batch(None, 1 << 18, 4) == N.C2G_ERR_INVALID
    ctx = Context(device=-1)
    for threads in (0, 32, 96, 512):
        assert lib.c2g_set_trace_block(ctx.handle, threads) == N.C2G_ERR_INVALID
    assert lib.c2g_set_trace_block(ctx.handle, 128) == N.C2G_ERR_STATE  # host-only: no device
    for records, windows in ((0, 4), (1023, 4), (1 << 18, 0), (1 << 18, 65)):
        assert lib.c2g_guide_batch(ctx.handle, records, windows) == N.C2G_ERR_INVALID
    assert lib.c2g_guide_batch(ctx.handle, 1 << 18, 4) == N.C2G_ERR_STATE
    for kappa, clamp, decay in ((0.5, 20.0, 0.0), (501.0, 20.0, 0.0), (100.0, 0.5, 0.0), (float("nan"), 20.0, 0.0),
                                (100.0, 10.0, -1.0)):
        assert lib.c2g_guide_regularize(ctx.handle, kappa, clamp, decay) == N.C2G_ERR_INVALID
    assert lib.c2g_guide_regularize(ctx.handle, 100.0, 10.0, 1000.0) == N.C2G_ERR_STATE
    # batch calls on a null batch
    assert lib.c2g_batch_set_lanes(None, 8) == N.C2G_ERR_INVALID
    assert lib.c2g_batch_set_trace(None, 4, 128) == N.C2G_ERR_INVALID
    assert lib.c2g_batch_search(None, None, 4, None) == N.C2G_ERR_INVALID
