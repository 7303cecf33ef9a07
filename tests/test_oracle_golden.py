"""The oracle port pinned against the reference's golden vectors (CPU only).

tests/golden/*.npz come from the reference renderer itself (tests/golden/make_goldens.py).
"""
import os

import numpy as np
import pytest

from crystal2_gb300 import scenes
from oracle import bindings as B

from golden_util import GOLDEN, SCENES, HALTON_RES, BSDF_PARAMS, bsdf_inputs, bsdf_kind


def test_halton_bits_match_reference():
    z = np.load(os.path.join(GOLDEN, "halton.npz"))
    for (W, H) in HALTON_RES:
        k = f"{W}x{H}"
        v = B.oracle_halton(W, H, z["px_" + k], z["py_" + k], z["s_" + k], 100)
        assert np.array_equal(v.view(np.uint32), z["bits_" + k]), k


@pytest.mark.parametrize("name", list(SCENES))
def test_bvh_order_and_nodes_match_reference(name, tmp_path):
    cp, sp = SCENES[name](str(tmp_path / name))
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, f"bvh_{name}.npz"))
    assert np.array_equal(o.bvh_order(), z["order"])
    b, a, ax = o.bvh_nodes()
    assert np.array_equal(b.view(np.uint32), z["bounds_bits"])
    assert np.array_equal(a, z["a"]) and np.array_equal(ax, z["axis"])


def test_camera_bits_match_reference(tmp_path):
    cp, sp = SCENES["cornell"](str(tmp_path / "c"))
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, "camera.npz"))
    co, cd = o.camera(z["pos"])
    assert np.array_equal(co.view(np.uint32), z["o_bits"])
    assert np.array_equal(cd.view(np.uint32), z["d_bits"])


@pytest.mark.parametrize("name", list(SCENES))
def test_intersections_match_reference(name, tmp_path):
    cp, sp = SCENES[name](str(tmp_path / name))
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, f"isect_{name}.npz"))
    obj, t = o.intersect(z["o"], z["d"])
    assert np.array_equal(obj, z["obj"])
    assert np.array_equal(t.view(np.uint32), z["t"].view(np.uint32))
    occ = o.intersect_test(z["o"], z["d"], z["tmin"], z["tmax"], z["ignore"])
    assert np.array_equal(occ, z["occ"])


def _phong_first_draw_accepted(frame, wo, u3, k, margin=1e-3):
    """Rows whose first Blinn-Phong half vector is clearly accepted (BlinnPhongReflection.cpp:36-50)."""
    N, T, Bv = (frame[i:i + 3].astype(np.float64) for i in (0, 3, 6))
    w = wo.astype(np.float64)
    wl = np.stack([w @ T, w @ N, w @ Bv], 1)
    ct = u3[:, 1].astype(np.float64) ** (1.0 / (k + 2))
    phi = 2 * np.pi * u3[:, 2].astype(np.float64)
    r = np.sqrt(np.maximum(0.0, 1 - ct * ct))
    h = np.stack([r * np.cos(phi), ct, -r * np.sin(phi)], 1)
    d = np.einsum("ij,ij->i", h, wl)
    refl_y = -wl[:, 1] + 2 * d * h[:, 1]
    return (d > margin) & (refl_y > margin)


def test_bsdf_matches_reference():
    z = np.load(os.path.join(GOLDEN, "bsdf.npz"))
    for k, (name, params) in enumerate(BSDF_PARAMS.items()):
        frame, wo, wi, u3 = bsdf_inputs(128, 100 + k)
        for front in (1, 0):
            for flags in (0x1F, 0x1F & ~8):
                fe, pe, fs, ws, ps, ts = B.bsdf_eval("orc", bsdf_kind(name), params, front, frame, wo, wi, u3, flags)
                key = f"{name}_{front}_{flags}"
                # identical float arithmetic except libm transcendentals: tight relative tolerance
                for got, want in ((fe, z[key + "_fe"]), (pe, z[key + "_pe"])):
                    np.testing.assert_allclose(got, want, rtol=2e-5, atol=1e-6, err_msg=key)
                first = _phong_first_draw_accepted(frame, wo, u3, params[8]) if name == "Phong" else slice(None)
                np.testing.assert_allclose(fs[first], z[key + "_fs"][first], rtol=2e-5, atol=1e-6, err_msg=key)
                # direction, pdf and type are defined only where the sample succeeded (f != 0)
                ok = np.any(z[key + "_fs"] != 0, axis=1)
                if name == "Phong":
                    # a rejected Blinn-Phong half vector is redrawn from the reference's shared
                    # std::mt19937 but from a hash here: compare first-draw acceptances only
                    ok &= _phong_first_draw_accepted(frame, wo, u3, params[8])
                np.testing.assert_allclose(ws[ok], z[key + "_ws"][ok], rtol=2e-5, atol=1e-6, err_msg=key)
                np.testing.assert_allclose(ps[ok], z[key + "_ps"][ok], rtol=2e-5, atol=1e-6, err_msg=key)
                assert np.array_equal(ts[ok], z[key + "_ts"][ok]), key


@pytest.mark.parametrize("name", ["cornell", "material_box", "spheres"])
def test_render_matches_reference(name, tmp_path):
    """Per-sample radiance is bit-identical to the reference's Evaluate for dims < 100 paths;
    the per-pixel mean image matches to float accumulation precision."""
    cp, sp = SCENES[name](str(tmp_path / name))
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    if name != "spheres":  # depth 12 paths reach dims >= 100, drawn from a different generator
        got = o.render_samples(z["px"], z["py"])
        assert np.array_equal(got.view(np.uint32), z["samples"].view(np.uint32))
        s, q, _ = o.render_region(0, 0, o.W, o.H)
        np.testing.assert_allclose(s / o.spp, z["mean"], rtol=1e-5, atol=1e-6)
    else:
        s, q, _ = o.render_region(0, 0, o.W, o.H)
        mean = s / o.spp
        var = np.maximum(z["m2"] - z["mean"] ** 2, 0) / o.spp + np.maximum(q / o.spp - mean ** 2, 0) / o.spp
        # statistically equal image means (3 standard errors of the difference)
        diff = (mean - z["mean"]).mean()
        se = np.sqrt(var.sum()) / mean.size
        assert abs(diff) <= 3 * se + 1e-6


def _direct_cornell(tmp_path):
    import json
    cp, sp = SCENES["cornell"](str(tmp_path / "direct"))
    cfg = json.load(open(cp))
    cfg["Integrator"]["Type"] = "DirectLight"
    json.dump(cfg, open(cp, "w"))
    return cp, sp


def test_direct_lighting_matches_reference(tmp_path):
    """DirectLightingIntegrator (DirectLightingIntegrator.cpp:22-156): bit-identical samples."""
    cp, sp = _direct_cornell(tmp_path)
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, "render_direct_cornell.npz"))
    got = o.render_samples(z["px"], z["py"])
    assert np.array_equal(got.view(np.uint32), z["samples"].view(np.uint32))
    s, q, _ = o.render_region(0, 0, o.W, o.H)
    np.testing.assert_allclose(s / o.spp, z["mean"], rtol=1e-5, atol=1e-6)


def test_brdf_box_render_matches_reference(tmp_path):
    """Oren-Nayar and Blinn-Phong materials (Reflections.cpp, BlinnPhongReflection.cpp): per-pixel
    means within 3 standard errors of the reference and most samples bit-identical (a rejected
    Blinn-Phong half vector is redrawn from a hash here, from a shared std::mt19937 there)."""
    cp, sp = scenes.brdf_box(str(tmp_path / "b"))
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, "render_brdf_box.npz"))
    s, q, _ = o.render_region(0, 0, o.W, o.H)
    mean = s / o.spp
    var = np.maximum(z["m2"] - z["mean"] ** 2, 0) / o.spp + np.maximum(q / o.spp - mean ** 2, 0) / o.spp
    assert abs((mean - z["mean"]).mean()) <= 3 * np.sqrt(var.sum()) / mean.size + 1e-6
    zt = (mean - z["mean"]) / np.sqrt(var + 1e-12)
    assert np.mean(np.abs(zt) > 3) <= 0.01
    got = o.render_samples(z["px"], z["py"])
    assert np.mean(got.view(np.uint32) == z["samples"].view(np.uint32)) >= 0.9


@pytest.mark.parametrize("integrator,name", [("PathTracer", "textured_yard"), ("DirectLight", "textured_yard_direct")])
def test_textured_render_matches_reference(tmp_path, integrator, name):
    """UV textures on a mesh, a sphere and a disk (Texel.cpp:15-19 nearest lookup with clamped,
    v-flipped uvs) and the cubemap skybox (CubemapTexture.cpp:24-58) seen by escaping rays: the
    oracle's per-pixel means match the reference's render and almost every sample is bit-identical
    (the Blinn-Phong disk may redraw a rejected half vector differently, see the brdf box)."""
    cp, sp = scenes.textured_yard(str(tmp_path / "t"), integrator=integrator)
    o = B.oracle_open(cp, sp)
    z = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    s, q, _ = o.render_region(0, 0, o.W, o.H)
    mean = s / o.spp
    var = np.maximum(z["m2"] - z["mean"] ** 2, 0) / o.spp + np.maximum(q / o.spp - mean ** 2, 0) / o.spp
    zt = (mean - z["mean"]) / np.sqrt(var + 1e-12)
    assert np.mean(np.abs(zt) > 3) <= 0.01
    assert np.mean(mean.astype(np.float32) == z["mean"]) >= 0.95
    got = o.render_samples(z["px"], z["py"])
    assert np.mean(got.view(np.uint32) == z["samples"].view(np.uint32)) >= 0.95


@pytest.mark.parametrize("name", ["sampler_default", "sampler_stratified", "sampler_default_direct"])
def test_oracle_samplers_match_reference_frames(tmp_path, name):
    """DefaultSampler and StratifiedSampler restated (a std::mt19937 per 32 x 32 tile seeded with
    the tile index, stratified tables filled and shuffled at StartPixel): the oracle's frame is the
    reference's SamplerIntegrator::Render frame to the bit."""
    from golden_util import sampler_scene
    cp, sp = sampler_scene(str(tmp_path), name)
    o = B.oracle_open(cp, sp)
    s, w = o.render_frame()
    z = np.load(os.path.join(GOLDEN, f"render_{name}.npz"))
    assert np.array_equal(w, z["weight"])
    assert np.array_equal(s.view(np.uint32), z["sum"].view(np.uint32))


@pytest.mark.parametrize("smp,spp", [("Stratified", 144), ("Default", 144)])
def test_per_draw_samplers_match_reference_streams_in_distribution(tmp_path, smp, spp):
    """The library draws Default / Stratified values per (pixel, sample, dimension); the reference
    advances one std::mt19937 per tile.  Both are estimators of the same image: 4 x 4-block means
    of the two (the reference's stream through the oracle, bit-exact to the reference's frames
    above) agree within 4 standard errors, and the image means within 3."""
    import json
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=40, height=36, spp=spp)
    cfg = json.load(open(cp))
    cfg["Integrator"]["Sampler"]["Type"] = smp
    json.dump(cfg, open(cp, "w"))
    o = B.oracle_open(cp, sp)
    res = []
    for counter in (False, True):
        o.set_counter_sampler(counter)
        s, q, _ = o.render_region(0, 0, o.W, o.H)
        m = s / spp
        res.append((m, np.maximum(q / spp - m ** 2, 0) / spp))

    def blocks(a):
        return a.reshape(9, 4, 10, 4, 3).mean(axis=(1, 3))
    (ma, va), (mb, vb) = res
    zt = (blocks(ma) - blocks(mb)) / np.sqrt((blocks(va) + blocks(vb)) / 16 + 1e-12)
    assert np.abs(zt).max() <= 4.0
    assert abs(ma.mean() - mb.mean()) <= 3 * np.sqrt((va + vb).sum()) / ma.size


def test_oracle_refuses_a_scene_without_objects(tmp_path):
    """An empty scene is an error for the oracle as for the library (the reference's BVH build
    crashes on it)."""
    cfg = scenes.config_json(13, 7, 2, 4)
    cp, sp = scenes.write_scene(str(tmp_path), cfg, scenes.camera((0, 0, -4), (0, 0, 0), 40), [], "empty")
    with pytest.raises(Exception):
        B.oracle_open(cp, sp)
