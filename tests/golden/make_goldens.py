#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ from the reference renderer itself.

The reference ships no tests or golden vectors for this path, so the fixtures are produced by
running the reference's own code (compiled from its sources by oracle/build_ref.py) on seeded
inputs.  Scene files are regenerated deterministically by crystal2_gb300.scenes, so only small
arrays are stored.  Run from the repository root with the reference tree available:

    python tests/golden/make_goldens.py

Fixtures:
  halton.npz     SampleValue bits for (pixel, sample, dims 0..99) at four film sizes
  camera.npz     GenerateRay origin/direction bits for 256 NDC points of the Cornell camera
  bvh_<scene>.npz  BVH::_objects order and node arrays (equal-count build)
  isect_<scene>.npz  Scene::Intersect (object, t) and Scene::IntersectTest results for seeded rays
  bsdf.npz       BSDF f/pdf and sampled (f, wi, pdf, type) for every material kind
  render_<scene>.npz per-sample radiance of a pixel subset and the per-pixel mean image
                 (cornell, material_box, spheres, direct_cornell, brdf_box: Oren-Nayar + Blinn-Phong,
                 textured_yard[_direct]: uv textures and the cubemap skybox; ``--only-textured``
                 regenerates just these two)
  render_sampler_*.npz  float frame sums and weights of SamplerIntegrator::Render with the Default
                 and Stratified samplers (``--only-samplers`` regenerates these and hdr_writer.npz)
  hdr_writer.npz stbi_write_hdr output bytes for synthetic float images
"""
from __future__ import annotations

import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from crystal2_gb300 import scenes  # noqa: E402
from oracle import bindings as B  # noqa: E402

# scene generators used by the fixtures (name -> callable(out_dir) -> (config, scene))
SCENES = {
    "cornell": lambda d: scenes.cornell(d, width=32, height=32, spp=16),
    "material_box": lambda d: scenes.material_box(d, width=32, height=32, spp=8),
    "soup": lambda d: scenes.tri_soup(d, n_tris=2000, seed=5, width=16, height=16),
    "spheres": lambda d: scenes.many_material(d, width=48, height=27, spp=4, n_grid=3, subdiv=1, depth=12),
}
HALTON_RES = [(32, 32), (256, 256), (1920, 1080), (100, 37)]


def ray_set(name: str, n: int, seed: int):
    rng = np.random.default_rng(seed)
    if name == "soup":
        return scenes.microbench_rays(n, seed, 256)
    lo = {"cornell": (-0.95, 0.05, -0.95), "material_box": (-1.9, 0.05, -1.9), "spheres": (-5, 0.1, -5)}[name]
    hi = {"cornell": (0.95, 1.95, 0.95), "material_box": (1.9, 2.9, 1.9), "spheres": (5, 3, 5)}[name]
    o = rng.uniform(lo, hi, size=(n, 3)).astype(np.float32)
    d = rng.normal(size=(n, 3))
    d /= np.linalg.norm(d, axis=1, keepdims=True)
    return o, d.astype(np.float32)


def anyhit_inputs(obj, t, n, seed):
    rng = np.random.default_rng(seed + 1)
    tt = np.where(np.isfinite(t), t, 4.0)
    tmax = (rng.random(n) * 2 * tt).astype(np.float32)
    tmin = np.zeros(n, np.float32)
    ign = np.where(rng.random(n) < 0.3, obj, -1).astype(np.int32)
    return tmin, tmax, ign


def bsdf_inputs(n: int, seed: int):
    rng = np.random.default_rng(seed)
    # frame: random orthonormal-ish (N, T, B) like a hit would have
    N = rng.normal(size=3); N /= np.linalg.norm(N)
    T = np.cross([1.0, 0, 0], N); T /= np.linalg.norm(T)
    Bv = np.cross(N, T)
    frame = np.concatenate([N, T, Bv]).astype(np.float32)
    wo = rng.normal(size=(n, 3)); wo /= np.linalg.norm(wo, axis=1, keepdims=True)
    wo = np.where((wo @ N)[:, None] < 0, -wo, wo)  # wo on the normal's side (the hit's N faces the ray)
    wi = rng.normal(size=(n, 3)); wi /= np.linalg.norm(wi, axis=1, keepdims=True)
    u3 = rng.random((n, 3))
    return frame, wo.astype(np.float32), wi.astype(np.float32), u3.astype(np.float32)


BSDF_PARAMS = {
    "Diffuse": [0.7, 0.5, 0.3, 0, 0, 0, 0, 0, 1],
    "Mirror": [0.9, 0.9, 0.8, 0, 0, 0, 0, 0, 1],
    "GlassRough": [1, 1, 1, 0, 0, 0, 0.1, 0.1, 1.5],
    "GlassSmooth": [1, 1, 1, 0, 0, 0, 0, 0, 1.5],
    "MicroGGX": [0.9, 0.7, 0.5, 0, 0, 0, 0.3, 0.3, 1.5],
    "MicroGGXAniso": [0.9, 0.7, 0.5, 0, 0, 0, 0.08, 0.45, 1.5],
    "MicroBeckmann": [0.8, 0.8, 0.8, 0, 0, 0, 0.25, 0.25, 1.5],
    "PlasticGGX": [0.5, 0.4, 0.3, 0.2, 0.2, 0.2, 0.3, 0.3, 1],
    "OrenNayar": [0.7, 0.6, 0.5, 0, 0, 0, 0, 0, 0.35],   # sigma in the last slot
    "Phong": [0.8, 0.7, 0.6, 0, 0, 0, 0, 0, 20],         # exponent K in the last slot
}


def bsdf_kind(name: str) -> str:
    return "MicroGGX" if name == "MicroGGXAniso" else name


def render_fixture(out: str, name: str, cp: str, sp: str, row_step: int = 5) -> None:
    """Mean and second moment of every pixel and the per-sample radiance of 16 pixels."""
    r = B.ref_open(cp, sp)
    s, q, _ = r.render_region(0, 0, r.W, r.H)
    px = np.arange(0, r.W, 3)[:16].astype(np.int32)
    py = ((np.arange(px.shape[0]) * row_step) % r.H).astype(np.int32)
    np.savez_compressed(os.path.join(out, f"render_{name}.npz"), mean=(s / r.spp).astype(np.float32),
                        m2=(q / r.spp).astype(np.float32), spp=r.spp, px=px, py=py, samples=r.render_samples(px, py))
    r.close()


def textured_goldens(out: str, work: str) -> None:
    """UV textures (Texel.cpp, UVTexture.h) and the cubemap skybox (CubemapTexture.cpp) under both
    integrators."""
    cp, sp = scenes.textured_yard(os.path.join(work, "textured_yard"))
    render_fixture(out, "textured_yard", cp, sp)
    cp, sp = scenes.textured_yard(os.path.join(work, "textured_yard_direct"), integrator="DirectLight")
    render_fixture(out, "textured_yard_direct", cp, sp)


SAMPLER_CASES = {  # fixture name -> (sampler, spp, integrator)
    "sampler_default": ("Default", 8, "PathTracer"),
    "sampler_stratified": ("Stratified", 9, "PathTracer"),
    "sampler_default_direct": ("Default", 8, "DirectLight"),
}


def sampler_scene(work: str, name: str):
    """The Cornell box at 40 x 36 with the case's sampler and integrator."""
    import json
    smp, spp, integ = SAMPLER_CASES[name]
    cp, sp = scenes.cornell(os.path.join(work, name), width=40, height=36, spp=spp)
    cfg = json.load(open(cp))
    cfg["Integrator"]["Sampler"]["Type"] = smp
    cfg["Integrator"]["Type"] = integ
    json.dump(cfg, open(cp, "w"))
    return cp, sp


def hdr_images():
    """Float images for the Radiance writer: widths below, inside and at the edges of the
    run-length range, zeros, tiny and huge values, and flat runs."""
    rng = np.random.default_rng(21)
    out = {}
    for w, h in ((5, 3), (8, 4), (64, 6), (300, 5)):
        a = rng.random((h, w, 3)).astype(np.float32) * np.float32(4.0)
        a[0, : w // 2] = 0.0
        a[1 % h, :] = np.float32(0.25)
        a[2 % h, w // 3:] = rng.choice(np.array([1e-35, 3e-10, 7.5, 65000.0, 1e20], np.float32), size=(w - w // 3, 3))
        out[f"{w}x{h}"] = a
    return out


def sampler_goldens(out: str, work: str) -> None:
    """DefaultSampler / StratifiedSampler frames (the reference's own SamplerIntegrator::Render
    into a FrameBuffer) and stbi_write_hdr files of synthetic images."""
    for name in SAMPLER_CASES:
        cp, sp = sampler_scene(work, name)
        r = B.ref_open(cp, sp)
        s, w, _ = r.render(threads=8)
        r.close()
        np.savez_compressed(os.path.join(out, f"render_{name}.npz"), sum=s, weight=w)
    Hz = {}
    for key, img in hdr_images().items():
        path = os.path.join(work, f"{key}.hdr")
        B.ref_write_hdr(path, img)
        Hz["img_" + key] = img
        Hz["file_" + key] = np.frombuffer(open(path, "rb").read(), np.uint8)
    np.savez_compressed(os.path.join(out, "hdr_writer.npz"), **Hz)


def main() -> None:
    out = HERE
    work = tempfile.mkdtemp(prefix="c2g_golden_")
    if "--only-textured" in sys.argv:
        textured_goldens(out, work)
        return
    if "--only-samplers" in sys.argv:
        sampler_goldens(out, work)
        return
    rng = np.random.default_rng(0)
    # Halton
    H = {}
    for (W, Hh) in HALTON_RES:
        n = 64
        px = rng.integers(0, W, n).astype(np.int32)
        py = rng.integers(0, Hh, n).astype(np.int32)
        s = rng.integers(0, 300, n).astype(np.int32)
        v = B.ref_halton(W, Hh, 1024, px, py, s, 100)
        H[f"px_{W}x{Hh}"], H[f"py_{W}x{Hh}"], H[f"s_{W}x{Hh}"] = px, py, s
        H[f"bits_{W}x{Hh}"] = v.view(np.uint32)
    np.savez_compressed(os.path.join(out, "halton.npz"), **H)
    # scenes: camera, BVH, intersections, renders
    for name, gen in SCENES.items():
        d = os.path.join(work, name)
        cp, sp = gen(d)
        r = B.ref_open(cp, sp)
        order = r.bvh_order()
        b, a, ax = r.bvh_nodes()
        np.savez_compressed(os.path.join(out, f"bvh_{name}.npz"), order=order, bounds_bits=b.view(np.uint32), a=a, axis=ax)
        n = 2000
        o, dd = ray_set(name, n, 11)
        obj, t = r.intersect(o, dd)
        tmin, tmax, ign = anyhit_inputs(obj, t, n, 11)
        occ = r.intersect_test(o, dd, tmin, tmax, ign)
        np.savez_compressed(os.path.join(out, f"isect_{name}.npz"), o=o, d=dd, obj=obj, t=t, tmin=tmin, tmax=tmax, ignore=ign, occ=occ)
        if name == "cornell":
            pos = rng.random((256, 2)).astype(np.float32)
            co, cd = r.camera(pos)
            np.savez_compressed(os.path.join(out, "camera.npz"), pos=pos, o_bits=co.view(np.uint32), d_bits=cd.view(np.uint32))
        if name in ("cornell", "material_box", "spheres"):
            W, Hh = r.W, r.H
            s, q, secs = r.render_region(0, 0, W, Hh)
            px = np.arange(0, W, 3)[:16].astype(np.int32)
            py = ((np.arange(px.shape[0]) * 7) % Hh).astype(np.int32)
            samples = r.render_samples(px, py)
            np.savez_compressed(os.path.join(out, f"render_{name}.npz"), mean=(s / r.spp).astype(np.float32),
                                m2=(q / r.spp).astype(np.float32), spp=r.spp, px=px, py=py, samples=samples)
        r.close()
    # direct lighting integrator (DirectLightingIntegrator.cpp) on the Cornell box
    import json
    d = os.path.join(work, "direct")
    cp, sp = SCENES["cornell"](d)
    cfg = json.load(open(cp))
    cfg["Integrator"]["Type"] = "DirectLight"
    json.dump(cfg, open(cp, "w"))
    r = B.ref_open(cp, sp)
    s, q, _ = r.render_region(0, 0, r.W, r.H)
    px = np.arange(0, r.W, 3)[:16].astype(np.int32)
    py = ((np.arange(px.shape[0]) * 5) % r.H).astype(np.int32)
    np.savez_compressed(os.path.join(out, "render_direct_cornell.npz"), mean=(s / r.spp).astype(np.float32),
                        m2=(q / r.spp).astype(np.float32), spp=r.spp, px=px, py=py, samples=r.render_samples(px, py))
    r.close()
    # Oren-Nayar and Blinn-Phong materials in a box (Reflections.cpp, BlinnPhongReflection.cpp)
    d = os.path.join(work, "brdf_box")
    cp, sp = scenes.brdf_box(d)
    r = B.ref_open(cp, sp)
    s, q, _ = r.render_region(0, 0, r.W, r.H)
    px = np.arange(0, r.W, 3)[:16].astype(np.int32)
    py = ((np.arange(px.shape[0]) * 5) % r.H).astype(np.int32)
    np.savez_compressed(os.path.join(out, "render_brdf_box.npz"), mean=(s / r.spp).astype(np.float32),
                        m2=(q / r.spp).astype(np.float32), spp=r.spp, px=px, py=py, samples=r.render_samples(px, py))
    r.close()
    # BSDFs
    Bz = {}
    for k, (name, params) in enumerate(BSDF_PARAMS.items()):
        frame, wo, wi, u3 = bsdf_inputs(128, 100 + k)
        for front in (1, 0):
            for flags in (0x1F, 0x1F & ~8):
                fe, pe, fs, ws, ps, ts = B.bsdf_eval("ref", bsdf_kind(name), params, front, frame, wo, wi, u3, flags)
                key = f"{name}_{front}_{flags}"
                Bz[key + "_fe"], Bz[key + "_pe"], Bz[key + "_fs"], Bz[key + "_ws"], Bz[key + "_ps"], Bz[key + "_ts"] = fe, pe, fs, ws, ps, ts
    np.savez_compressed(os.path.join(out, "bsdf.npz"), **Bz)
    textured_goldens(out, work)
    sampler_goldens(out, work)
    print("goldens written to", out)


if __name__ == "__main__":
    main()
