"""Seeded synthetic scenes in the reference's own input format (config JSON + scene JSON + OBJ).

Both engines read the same files, so every parity comparison starts from identical inputs.  The
reference ships scenes whose OBJ models are absent, so the workloads are generated here:

* ``cornell``        Cornell-style box (10 triangles), a diffuse and a mirror sphere, a 0.5 x 0.5
                     ceiling light of radiance 15; 256^2, 64 spp, depth 8, Halton, BVH.
* ``material_box``   small box exercising every material, both light kinds and a pass-through
                     object (parity of the BSDF/light code at low resolution).
* ``tri_soup``       1M random triangles in the unit cube (ray-intersection microbenchmark) and its
                     16M-ray set (``microbench_rays``).
* ``many_material``  400 subdivision-4 icospheres (5120 triangles each) on a jittered 20 x 20 grid
                     over a 40 x 40 ground quad, five material families, two area quads of radiance
                     20 and a point light of intensity 50; 1920 x 1080, 256 spp, depth 16.
* ``textured_yard``  UV-textured floor quad, sphere and disk (Diffuse and Phong ``Kd`` textures),
                     an area light, a point light and a six-face skybox; textures are binary PPM.
* ``slit_room``      closed 10 x 4 x 10 room lit through a 0.2-wide slit by an exterior 2 x 2 light
                     of radiance 200; 512 x 512 value-noise heightfield floor; GGX everywhere.

Numbers written to JSON use at most 6 significant digits; OBJ coordinates are float32 values
printed with 9 significant digits, which round-trip exactly through sscanf("%lf") -> float.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np


# ---- writers ---------------------------------------------------------------------------------

def _f(x: float) -> float:
    """Round a JSON number to 6 significant digits (both JSON readers then see the same text)."""
    return float(f"{float(x):.6g}")


def _v(v) -> list:
    return [_f(c) for c in v]


def write_obj(path: str, V: np.ndarray, N: np.ndarray, F: np.ndarray, FN: np.ndarray | None = None) -> None:
    """Triangles F (m,3, 0-based) over positions V and normals N; FN indexes N (default F)."""
    V = np.asarray(V, dtype=np.float32)
    N = np.asarray(N, dtype=np.float32)
    F = np.asarray(F, dtype=np.int64) + 1
    FN = F if FN is None else np.asarray(FN, dtype=np.int64) + 1
    with open(path, "w") as fh:
        fh.write("\n".join("v %.9g %.9g %.9g" % tuple(r) for r in V.tolist()))
        fh.write("\n")
        fh.write("\n".join("vn %.9g %.9g %.9g" % tuple(r) for r in N.tolist()))
        fh.write("\n")
        ff = np.stack([F[:, 0], FN[:, 0], F[:, 1], FN[:, 1], F[:, 2], FN[:, 2]], axis=1)
        fh.write("\n".join("f %d//%d %d//%d %d//%d" % tuple(r) for r in ff.tolist()))
        fh.write("\n")


def write_obj_uv(path: str, V, N, T, F) -> None:
    """Triangles F (m,3, 0-based) that index positions V, texture coordinates T and normals N alike."""
    V = np.asarray(V, dtype=np.float32)
    N = np.asarray(N, dtype=np.float32)
    T = np.asarray(T, dtype=np.float32)
    F = np.asarray(F, dtype=np.int64) + 1
    with open(path, "w") as fh:
        for r in V.tolist():
            fh.write("v %.9g %.9g %.9g\n" % tuple(r))
        for r in T.tolist():
            fh.write("vt %.9g %.9g\n" % tuple(r))
        for r in N.tolist():
            fh.write("vn %.9g %.9g %.9g\n" % tuple(r))
        for r in F.tolist():
            fh.write("f %d/%d/%d %d/%d/%d %d/%d/%d\n" % (r[0], r[0], r[0], r[1], r[1], r[1], r[2], r[2], r[2]))


def write_ppm(path: str, rgb) -> None:
    """Binary PPM (P6, maxval 255) of an (h, w, 3) uint8 array; row 0 is the top of the image."""
    rgb = np.ascontiguousarray(rgb, dtype=np.uint8)
    h, w, _ = rgb.shape
    with open(path, "wb") as fh:
        fh.write(b"P6\n%d %d\n255\n" % (w, h))
        fh.write(rgb.tobytes())


def quad_obj(path: str, corners, normal) -> None:
    """Two triangles (0,1,2) and (0,2,3) over four corners with one face normal."""
    V = np.asarray(corners, dtype=np.float32)
    N = np.asarray([normal], dtype=np.float32)
    F = np.array([[0, 1, 2], [0, 2, 3]])
    write_obj(path, V, N, F, FN=np.zeros_like(F))


def config_json(width, height, spp, depth, accel="BVH", integrator="PathTracer", threads=8, sampler="Halton", seed=0) -> dict:
    return {"Width": int(width), "Height": int(height), "SamplesPerPixel": int(spp), "Threads": int(threads),
            "Acceleration": accel,
            "Integrator": {"Type": integrator, "Depth": int(depth), "Sampler": {"Type": sampler, "Seed": int(seed)}}}


def mesh(obj_path: str, material: dict | None, translation=(0, 0, 0), scale=(1, 1, 1), rotation=(0, 0, 0), area_light=None) -> dict:
    o = {"Type": "Geometry", "Shape": {"Type": "TriangleMesh", "ObjFile": obj_path, "Translation": _v(translation),
                                        "Scale": _v(scale), "Rotation": _v(rotation)}}
    if material is not None:
        o["Material"] = material
    if area_light is not None:
        o["AreaLight"] = {"Type": "Diffused", "Lemit": _v(area_light), "Samples": 1}
    return o


def sphere(pos, r, material: dict | None, rotation=None, area_light=None) -> dict:
    o = {"Type": "Geometry", "Shape": {"Type": "Sphere", "Position": _v(pos), "Radius": _f(r)}}
    if rotation is not None:
        o["Shape"]["Rotation"] = _v(rotation)
    if material is not None:
        o["Material"] = material
    if area_light is not None:
        o["AreaLight"] = {"Type": "Diffused", "Lemit": _v(area_light), "Samples": 1}
    return o


def disk(pos, r, material: dict | None, rotation=(0, 0, 0), area_light=None) -> dict:
    o = {"Type": "Geometry", "Shape": {"Type": "Disk", "Position": _v(pos), "Radius": _f(r), "Rotation": _v(rotation)}}
    if material is not None:
        o["Material"] = material
    if area_light is not None:
        o["AreaLight"] = {"Type": "Diffused", "Lemit": _v(area_light), "Samples": 1}
    return o


def diffuse(c) -> dict:
    return {"Type": "Diffuse", "Color": _v(c)}


def mirror(c=(1, 1, 1)) -> dict:
    return {"Type": "Mirror", "Color": _v(c)}


def micro(c, ax, ay=None, ndf="GGX", ior=1.5) -> dict:
    return {"Type": "Micro", "Color": _v(c), "Roughness": [_f(ax), _f(ax if ay is None else ay)], "IOR": _f(ior), "NDF": ndf}


def glass(c=(1, 1, 1), rough=(0.1, 0.1), ior=1.5) -> dict:
    return {"Type": "Glass", "Color": _v(c), "Roughness": _v(rough), "IOR": _f(ior)}


def oren_nayar(c, sigma) -> dict:
    return {"Type": "OrenNayar", "Color": _v(c), "Sigma": _f(sigma)}


def phong(c, k: int) -> dict:
    return {"Type": "Phong", "Color": _v(c), "K": int(k)}


def plastic(kd, ks, rough, ndf="GGX") -> dict:
    return {"Type": "Plastic", "Kd": _v(kd), "Ks": _v(ks), "Roughness": _v(rough), "NDF": ndf}


def camera(pos, look_at, fov, up=(0, 1, 0)) -> dict:
    return {"Type": "Normal", "Position": _v(pos), "LookAt": _v(look_at), "Up": _v(up), "FOV": _f(fov)}


def point_light(pos, flux) -> dict:
    return {"Type": "Light", "LightType": "Point", "Position": _v(pos), "Flux": _v(flux)}


def diffuse_tex(name: str) -> dict:
    return {"Type": "Diffuse", "Kd": name}


def phong_tex(name: str, k: int) -> dict:
    return {"Type": "Phong", "Kd": name, "K": int(k)}


def write_scene(out_dir: str, cfg: dict, cam: dict, objects: list, name: str = "scene",
                textures: dict | None = None, skybox: str | None = None) -> tuple[str, str]:
    """textures: name -> image path (the scene's "Textures"); skybox: folder of the six faces."""
    os.makedirs(out_dir, exist_ok=True)
    cpath = os.path.join(out_dir, f"{name}_config.json")
    spath = os.path.join(out_dir, f"{name}.json")
    with open(cpath, "w") as fh:
        json.dump(cfg, fh, indent=1)
    sc = {"Textures": {k: {"Path": v} for k, v in (textures or {}).items()}, "Objects": objects}
    if skybox is not None:
        sc["Skybox"] = {"Path": skybox}
    with open(spath, "w") as fh:
        json.dump({"Camera": cam, "Scene": sc}, fh, indent=1)
    return cpath, spath


# ---- Cornell box -----------------------------------------------------------------------------

def _box_walls(d: str, x0=-1.0, x1=1.0, y0=0.0, y1=2.0, z0=-1.0, z1=1.0) -> dict:
    """Floor, ceiling, back, +x and -x walls (inward normals) as OBJ files; returns name -> path."""
    walls = {
        "floor": ([(x0, y0, z0), (x1, y0, z0), (x1, y0, z1), (x0, y0, z1)], (0, 1, 0)),
        "ceiling": ([(x0, y1, z0), (x0, y1, z1), (x1, y1, z1), (x1, y1, z0)], (0, -1, 0)),
        "back": ([(x0, y0, z1), (x1, y0, z1), (x1, y1, z1), (x0, y1, z1)], (0, 0, -1)),
        "xpos": ([(x1, y0, z0), (x1, y1, z0), (x1, y1, z1), (x1, y0, z1)], (-1, 0, 0)),
        "xneg": ([(x0, y0, z0), (x0, y0, z1), (x0, y1, z1), (x0, y1, z0)], (1, 0, 0)),
    }
    out = {}
    for name, (corners, n) in walls.items():
        p = os.path.join(d, f"{name}.obj")
        quad_obj(p, corners, n)
        out[name] = p
    return out


def cornell(out_dir: str, width=256, height=256, spp=64, depth=8, accel="BVH", threads=8) -> tuple[str, str]:
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    w = _box_walls(d)
    lp = os.path.join(d, "light.obj")
    h, ly = 0.25, 1.999
    quad_obj(lp, [(-h, ly, -h), (-h, ly, h), (h, ly, h), (h, ly, -h)], (0, -1, 0))
    white, red, green = (0.73, 0.73, 0.73), (0.65, 0.05, 0.05), (0.12, 0.45, 0.15)
    objs = [
        mesh(w["floor"], diffuse(white)),
        mesh(w["ceiling"], diffuse(white)),
        mesh(w["back"], diffuse(white)),
        mesh(w["xpos"], diffuse(red)),     # image left (camera right vector is -x)
        mesh(w["xneg"], diffuse(green)),
        mesh(lp, diffuse((0, 0, 0)), area_light=(15, 15, 15)),
        sphere((-0.45, 0.3, 0.25), 0.3, diffuse(white)),
        sphere((0.45, 0.3, -0.3), 0.3, mirror((1, 1, 1))),
    ]
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads)
    return write_scene(d, cfg, camera((0, 1, -3.8), (0, 1, 0), 40), objs, "cornell")


def cornell_variant(out_dir: str, seed: int, width=256, height=256, spp=64, depth=8, accel="BVH",
                    threads=8) -> tuple[str, str]:
    """The Cornell box with its materials re-drawn from `seed`: wall albedos U(0.2, 0.9) per channel,
    the two spheres each diffuse, GGX (alpha U(0.05, 0.6)) or mirror."""
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    w = _box_walls(d)
    lp = os.path.join(d, "light.obj")
    h, ly = 0.25, 1.999
    quad_obj(lp, [(-h, ly, -h), (-h, ly, h), (h, ly, h), (h, ly, -h)], (0, -1, 0))

    def ball():
        k = int(rng.integers(0, 3))
        if k == 0:
            return diffuse(rng.uniform(0.2, 0.9, 3))
        if k == 1:
            return micro(rng.uniform(0.5, 1.0, 3), rng.uniform(0.05, 0.6))
        return mirror(rng.uniform(0.7, 1.0, 3))

    objs = [mesh(w[k], diffuse(rng.uniform(0.2, 0.9, 3))) for k in ("floor", "ceiling", "back", "xpos", "xneg")]
    objs += [mesh(lp, diffuse((0, 0, 0)), area_light=(15, 15, 15)),
             sphere((-0.45, 0.3, 0.25), 0.3, ball()), sphere((0.45, 0.3, -0.3), 0.3, ball())]
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads)
    return write_scene(d, cfg, camera((0, 1, -3.8), (0, 1, 0), 40), objs, "cornell")


def batch_jobs(out_dir: str, n_jobs: int = 64, seed: int = 4, n_grid: int = 8, subdiv: int = 4):
    """Seeded multi-job workload: each job a variant of the Cornell box or of the many-material
    scene (materials re-drawn; the many-material variant on an n_grid x n_grid sphere grid),
    square resolution log-uniform in [128, 1024], spp from {16, 64, 256, 1024}, guided or plain.
    Returns [(config_path, scene_path, spp, guided)]."""
    rng = np.random.default_rng(seed)
    jobs = []
    for j in range(n_jobs):
        side = int(round(2 ** rng.uniform(7, 10)))
        spp = int(rng.choice([16, 64, 256, 1024]))
        guided = bool(rng.integers(0, 2))
        d = os.path.join(out_dir, f"job{j:03d}")
        if rng.integers(0, 2) == 0:
            cp, sp = cornell_variant(d, seed=1000 + j, width=side, height=side, spp=spp)
        else:
            cp, sp = many_material(d, width=side, height=side, spp=spp, seed=2000 + j, n_grid=n_grid, subdiv=subdiv)
        jobs.append((cp, sp, spp, guided))
    return jobs


def brdf_box(out_dir: str, width=48, height=48, spp=16, depth=6, accel="BVH", threads=8) -> tuple[str, str]:
    """Box with Oren-Nayar walls (sigma 0.3 / 0.7) and Blinn-Phong spheres (K 8 and 60)."""
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    w = _box_walls(d)
    lp = os.path.join(d, "light.obj")
    h, ly = 0.3, 1.999
    quad_obj(lp, [(-h, ly, -h), (-h, ly, h), (h, ly, h), (h, ly, -h)], (0, -1, 0))
    objs = [
        mesh(w["floor"], oren_nayar((0.7, 0.7, 0.7), 0.3)),
        mesh(w["ceiling"], oren_nayar((0.75, 0.75, 0.75), 0.7)),
        mesh(w["back"], oren_nayar((0.6, 0.6, 0.7), 0.5)),
        mesh(w["xpos"], oren_nayar((0.65, 0.1, 0.1), 0.7)),
        mesh(w["xneg"], diffuse((0.1, 0.5, 0.15))),
        mesh(lp, diffuse((0, 0, 0)), area_light=(14, 14, 14)),
        sphere((-0.45, 0.35, 0.2), 0.35, phong((0.8, 0.8, 0.8), 8)),
        sphere((0.45, 0.3, -0.25), 0.3, phong((0.9, 0.7, 0.4), 60)),
    ]
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads)
    return write_scene(d, cfg, camera((0, 1, -3.8), (0, 1, 0), 40), objs, "brdf_box")


def textured_yard(out_dir: str, width=64, height=48, spp=16, depth=6, accel="BVH", threads=8, seed=5,
                  integrator="PathTracer", skybox=True) -> tuple[str, str]:
    """Open scene for the texture and skybox paths: a 4 x 4 floor quad whose uvs run from -0.1 to 1.1
    (the texel lookup clamps), a sphere and a disk with Diffuse / Phong ``Kd`` textures, a 1 x 1 area
    light, a point light, and a six-face skybox seen above the horizon.  Textures are seeded random
    binary PPM images; the faces are named ``posx.jpg`` ... ``negz.jpg`` as the scene format expects
    (both loaders detect PPM by content)."""
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    checker = np.kron((np.indices((8, 8)).sum(0) % 2)[..., None], np.ones((2, 2, 1)))  # 16 x 16
    ca, cb = rng.integers(40, 250, 3), rng.integers(10, 120, 3)
    write_ppm(os.path.join(d, "floor.ppm"), np.where(checker > 0, ca, cb))
    write_ppm(os.path.join(d, "noise.ppm"), rng.integers(0, 256, (24, 32, 3)))
    ramp = np.linspace(20, 235, 16)
    write_ppm(os.path.join(d, "ramp.ppm"), np.stack([np.tile(ramp, (12, 1)), np.tile(ramp[:12, None], (1, 16)),
                                                     np.full((12, 16), 90.0)], axis=-1))
    sky = os.path.join(d, "sky")
    os.makedirs(sky, exist_ok=True)
    for k, face in enumerate(("posx", "negx", "posy", "negy", "posz", "negz")):
        tint = np.array([60 + 30 * k, 200 - 25 * k, 120 + 15 * (k % 3)])
        img = np.clip(tint + rng.integers(-40, 40, (8, 8, 3)), 0, 255)
        write_ppm(os.path.join(sky, face + ".jpg"), img)
    fp = os.path.join(d, "floor.obj")
    write_obj_uv(fp, [(-2, 0, -1), (2, 0, -1), (2, 0, 3), (-2, 0, 3)], [(0, 1, 0)] * 4,
                 [(-0.1, -0.1), (1.1, -0.1), (1.1, 1.1), (-0.1, 1.1)], [[0, 2, 1], [0, 3, 2]])
    lp = os.path.join(d, "light.obj")
    quad_obj(lp, [(-0.5, 2.5, 0.5), (-0.5, 2.5, 1.5), (0.5, 2.5, 1.5), (0.5, 2.5, 0.5)], (0, -1, 0))
    objs = [
        mesh(fp, diffuse_tex("floor")),
        sphere((-0.6, 0.5, 1.0), 0.5, diffuse_tex("noise"), rotation=(0, 35, 0)),
        disk((0.8, 0.6, 1.2), 0.5, phong_tex("ramp", 12), rotation=(-70, 20, 0)),
        mesh(lp, diffuse((0, 0, 0)), area_light=(6, 6, 6)),
        point_light((1.5, 1.8, -0.5), (3, 3, 3)),
    ]
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads, integrator=integrator)
    tex = {"floor": os.path.join(d, "floor.ppm"), "noise": os.path.join(d, "noise.ppm"),
           "ramp": os.path.join(d, "ramp.ppm")}
    return write_scene(d, cfg, camera((0, 1.0, -2.5), (0, 0.7, 1.0), 60), objs, "textured_yard",
                       textures=tex, skybox=sky if skybox else None)


def material_box(out_dir: str, width=64, height=64, spp=16, depth=8, accel="BVH", threads=8) -> tuple[str, str]:
    """Every material family, a disk, a point light, a sphere light and a pass-through object."""
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    w = _box_walls(d, -2, 2, 0, 3, -2, 2)
    lp = os.path.join(d, "light.obj")
    quad_obj(lp, [(-0.4, 2.99, -0.4), (-0.4, 2.99, 0.4), (0.4, 2.99, 0.4), (0.4, 2.99, -0.4)], (0, -1, 0))
    panel = os.path.join(d, "panel.obj")
    quad_obj(panel, [(-1.8, 0.2, 1.2), (-1.8, 1.4, 1.2), (-1.0, 1.4, 1.2), (-1.0, 0.2, 1.2)], (0, 0, -1))
    objs = [
        mesh(w["floor"], plastic((0.5, 0.4, 0.3), (0.2, 0.2, 0.2), (0.3, 0.3))),
        mesh(w["ceiling"], diffuse((0.8, 0.8, 0.8))),
        mesh(w["back"], micro((0.9, 0.8, 0.7), 0.3, ndf="Beckmann")),
        mesh(w["xpos"], diffuse((0.7, 0.1, 0.1))),
        mesh(w["xneg"], diffuse((0.1, 0.6, 0.2))),
        mesh(lp, None, area_light=(12, 12, 12)),                       # pass-through emitter
        mesh(panel, None),                                             # pass-through panel
        sphere((-1.0, 0.5, 0.0), 0.5, micro((0.9, 0.9, 0.9), 0.2)),
        sphere((0.2, 0.45, 0.6), 0.45, micro((0.95, 0.7, 0.4), 0.08, 0.4), rotation=(0, 30, 0)),
        sphere((1.1, 0.5, -0.3), 0.5, glass((1, 1, 1), (0.1, 0.1), 1.5)),
        sphere((0.0, 0.35, -0.9), 0.35, mirror((0.9, 0.9, 0.9))),
        sphere((1.3, 1.6, 1.0), 0.25, glass((1, 1, 1), (0.0, 0.0), 1.5)),
        sphere((-1.4, 2.3, 1.4), 0.15, diffuse((0, 0, 0)), area_light=(20, 16, 12)),
        disk((0.8, 0.01, 1.2), 0.4, diffuse((0.3, 0.3, 0.8)), rotation=(0, 0, 0)),
        disk((-0.5, 2.0, 1.99), 0.3, diffuse((0, 0, 0)), rotation=(-90, 0, 0), area_light=(6, 6, 9)),
        point_light((1.5, 2.5, -1.5), (40, 40, 40)),
    ]
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads)
    return write_scene(d, cfg, camera((0, 1.5, -5.5), (0, 1.2, 0), 45), objs, "material_box")


# ---- triangle soup (ray microbenchmark) ------------------------------------------------------

def tri_soup_arrays(n_tris: int, seed: int = 1) -> np.ndarray:
    """(n, 3, 3) float32: centroids ~U[0,1]^3, each vertex = centroid + U(-0.005, 0.005)^3."""
    rng = np.random.default_rng(seed)
    c = rng.random((n_tris, 1, 3), dtype=np.float64)
    v = c + rng.uniform(-0.005, 0.005, size=(n_tris, 3, 3))
    return v.astype(np.float32)


def tri_soup(out_dir: str, n_tris: int = 1 << 20, seed: int = 1, width=64, height=64) -> tuple[str, str]:
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    tris = tri_soup_arrays(n_tris, seed)
    e1 = tris[:, 1] - tris[:, 0]
    e2 = tris[:, 2] - tris[:, 0]
    n = np.cross(e1.astype(np.float64), e2.astype(np.float64))
    n /= np.maximum(np.linalg.norm(n, axis=1, keepdims=True), 1e-30)
    V = tris.reshape(-1, 3)
    F = np.arange(3 * n_tris).reshape(-1, 3)
    FN = np.repeat(np.arange(n_tris)[:, None], 3, axis=1)
    p = os.path.join(d, "soup.obj")
    write_obj(p, V, n.astype(np.float32), F, FN)
    objs = [mesh(p, diffuse((0.5, 0.5, 0.5)))]
    cfg = config_json(width, height, 1, 4)
    return write_scene(d, cfg, camera((0.5, 0.5, -1.5), (0.5, 0.5, 0.5), 45), objs, "soup")


def microbench_rays(n_rays: int, seed: int = 1, res: int = 4096):
    """Half coherent pinhole primaries (res x res image of the unit cube), half incoherent rays
    with origins ~U[0,1]^3 and directions uniform on the sphere.  Returns (o, d) float32 (n,3)."""
    rng = np.random.default_rng(seed + 17)
    n0 = n_rays // 2
    n1 = n_rays - n0
    eye = np.array([0.5, 0.5, -1.5])
    look = np.array([0.0, 0.0, 1.0])
    right = np.array([-1.0, 0.0, 0.0])
    up = np.array([0.0, 1.0, 0.0])
    th = math.tan(math.radians(45) / 2)
    idx = np.arange(n0)
    stride = max(1, (res * res) // max(1, n0))
    pix = (idx * stride) % (res * res)
    px = (pix % res + 0.5) / res * 2 - 1
    py = (pix // res + 0.5) / res * 2 - 1
    dirs = right[None] * (px[:, None] * th) + up[None] * (py[:, None] * th) + look[None]
    dirs /= np.linalg.norm(dirs, axis=1, keepdims=True)
    o0 = np.repeat(eye[None], n0, axis=0)
    o1 = rng.random((n1, 3))
    z = rng.uniform(-1, 1, n1)
    phi = rng.uniform(0, 2 * math.pi, n1)
    r = np.sqrt(1 - z * z)
    d1 = np.stack([r * np.cos(phi), z, r * np.sin(phi)], axis=1)
    o = np.concatenate([o0, o1]).astype(np.float32)
    dd = np.concatenate([dirs, d1]).astype(np.float32)
    return np.ascontiguousarray(o), np.ascontiguousarray(dd)


# ---- icospheres / many-material scene ----------------------------------------------------------

def icosphere(subdiv: int = 4):
    """Unit icosphere: vertices (unit length, float64) and faces (outward winding)."""
    t = (1 + 5 ** 0.5) / 2
    V = [(-1, t, 0), (1, t, 0), (-1, -t, 0), (1, -t, 0), (0, -1, t), (0, 1, t), (0, -1, -t), (0, 1, -t),
         (t, 0, -1), (t, 0, 1), (-t, 0, -1), (-t, 0, 1)]
    V = [np.array(v, dtype=np.float64) / np.linalg.norm(v) for v in V]
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4), (11, 10, 2), (10, 7, 6),
         (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8), (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10),
         (8, 6, 7), (9, 8, 1)]
    for _ in range(subdiv):
        cache = {}
        nf = []

        def mid(a, b):
            k = (min(a, b), max(a, b))
            if k not in cache:
                m = V[a] + V[b]
                V.append(m / np.linalg.norm(m))
                cache[k] = len(V) - 1
            return cache[k]

        for a, b, c in F:
            ab, bc, ca = mid(a, b), mid(b, c), mid(c, a)
            nf += [(a, ab, ca), (b, bc, ab), (c, ca, bc), (ab, bc, ca)]
        F = nf
    return np.array(V), np.array(F)


def many_material(out_dir: str, width=1920, height=1080, spp=256, depth=16, seed=2, n_grid=20, subdiv=4,
                  accel="BVH", threads=16) -> tuple[str, str]:
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    V, F = icosphere(subdiv)
    ico = os.path.join(d, f"ico{subdiv}.obj")
    write_obj(ico, V.astype(np.float32), V.astype(np.float32), F)
    ground = os.path.join(d, "ground.obj")
    quad_obj(ground, [(-20, 0, -20), (-20, 0, 20), (20, 0, 20), (20, 0, -20)], (0, 1, 0))
    objs = [mesh(ground, diffuse((0.6, 0.6, 0.6)))]
    spacing = 40.0 / n_grid
    for i in range(n_grid):
        for j in range(n_grid):
            r = rng.uniform(0.2, 0.5)
            cx = -20 + spacing * (i + 0.5) + rng.uniform(-0.3, 0.3) * spacing
            cz = -20 + spacing * (j + 0.5) + rng.uniform(-0.3, 0.3) * spacing
            kind = int(rng.integers(0, 5))
            if kind == 0:
                m = micro(rng.uniform(0.5, 1.0, 3), rng.uniform(0.05, 0.8))
            elif kind == 1:
                m = micro(rng.uniform(0.5, 1.0, 3), rng.uniform(0.05, 0.6), rng.uniform(0.05, 0.6))
            elif kind == 2:
                m = glass((1, 1, 1), (0.1, 0.1), 1.5)
            elif kind == 3:
                m = mirror(rng.uniform(0.7, 1.0, 3))
            else:
                m = diffuse(rng.uniform(0.2, 0.9, 3))
            objs.append(mesh(ico, m, translation=(cx, r, cz), scale=(r, r, r)))
    for lx in (-8.0, 8.0):
        lp = os.path.join(d, f"arealight_{int(lx)}.obj")
        quad_obj(lp, [(lx - 2, 12, -2), (lx - 2, 12, 2), (lx + 2, 12, 2), (lx + 2, 12, -2)], (0, -1, 0))
        objs.append(mesh(lp, diffuse((0, 0, 0)), area_light=(20, 20, 20)))
    objs.append(point_light((0, 10, -8), [50 * 4 * math.pi] * 3))
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads)
    return write_scene(d, cfg, camera((0, 9, -28), (0, 0, 0), 45), objs, "many_material")


# ---- slit-lit room with a heightfield floor ----------------------------------------------------

def _value_noise(res: int, rng, octaves=4, amplitude=0.3) -> np.ndarray:
    h = np.zeros((res, res))
    x = np.linspace(0, 1, res)
    for o in range(octaves):
        cells = 4 * (2 ** o)
        g = rng.random((cells + 1, cells + 1))
        fx = x * cells
        i0 = np.minimum(fx.astype(int), cells - 1)
        t = fx - i0
        t = t * t * (3 - 2 * t)
        a = g[i0][:, i0]
        b = g[i0 + 1][:, i0]
        c = g[i0][:, i0 + 1]
        dd = g[i0 + 1][:, i0 + 1]
        tx = t[None, :]
        ty = t[:, None]
        v = (a * (1 - ty) + b * ty) * (1 - tx) + (c * (1 - ty) + dd * ty) * tx
        h += v / (2 ** o)
    h -= h.min()
    h /= max(h.max(), 1e-9)
    return h * amplitude


def heightfield_obj(path: str, res: int, half: float, rng, amplitude=0.3) -> None:
    H = _value_noise(res, rng, amplitude=amplitude)
    xs = np.linspace(-half, half, res)
    X, Z = np.meshgrid(xs, xs, indexing="xy")
    V = np.stack([X, H, Z], axis=-1).reshape(-1, 3)
    # smooth normals from central differences
    dhx = np.gradient(H, xs, axis=1)
    dhz = np.gradient(H, xs, axis=0)
    N = np.stack([-dhx, np.ones_like(H), -dhz], axis=-1).reshape(-1, 3)
    N /= np.linalg.norm(N, axis=1, keepdims=True)
    idx = np.arange(res * res).reshape(res, res)
    a = idx[:-1, :-1].ravel()
    b = idx[:-1, 1:].ravel()
    c = idx[1:, 1:].ravel()
    dd = idx[1:, :-1].ravel()
    F = np.concatenate([np.stack([a, dd, c], 1), np.stack([a, c, b], 1)])
    write_obj(path, V.astype(np.float32), N.astype(np.float32), F)


def slit_room(out_dir: str, width=1920, height=1080, spp=64, depth=12, seed=3, hf_res=512, accel="Brute",
              threads=16, integrator="PathTracer") -> tuple[str, str]:
    """Closed 10 x 4 x 10 room lit only through a 0.2-wide slit in the back wall by an exterior 2 x 2
    area light of radiance 200; 512 x 512 heightfield floor (4-octave value noise, amplitude 0.3);
    every surface GGX with alpha U(0.1, 0.3).

    The default accelerator is "Brute" (exact any-hit semantics; this library traverses the same SAH
    tree for both names).  The reference's BVH shadow test clips the ray interval to each object's
    box and lets shadow rays through axis-aligned walls whose planes are not exactly representable
    (BVH.cpp:132-134): here that leak lights the room about 3x brighter than the slit does, and the
    scene exists to test occlusion by a wall."""
    d = os.path.abspath(out_dir)
    os.makedirs(d, exist_ok=True)
    rng = np.random.default_rng(seed)
    hx, hy, hz = 5.0, 4.0, 5.0
    hf = os.path.join(d, f"heightfield{hf_res}.obj")
    heightfield_obj(hf, hf_res, hx, rng)

    def rough():
        return micro(rng.uniform(0.5, 0.9, 3), rng.uniform(0.1, 0.3))

    objs = [mesh(hf, rough())]
    quads = {
        "ceiling": ([(-hx, hy, -hz), (-hx, hy, hz), (hx, hy, hz), (hx, hy, -hz)], (0, -1, 0)),
        "front": ([(-hx, 0, -hz), (-hx, hy, -hz), (hx, hy, -hz), (hx, 0, -hz)], (0, 0, 1)),
        "xpos": ([(hx, 0, -hz), (hx, hy, -hz), (hx, hy, hz), (hx, 0, hz)], (-1, 0, 0)),
        "xneg": ([(-hx, 0, -hz), (-hx, 0, hz), (-hx, hy, hz), (-hx, hy, -hz)], (1, 0, 0)),
    }
    # back wall (z = +hz) with a horizontal 0.2-wide slit at y in [2.9, 3.1], x in [-3, 3]
    s0, s1, sx = 2.9, 3.1, 3.0
    back = [
        ([(-hx, 0, hz), (hx, 0, hz), (hx, s0, hz), (-hx, s0, hz)]),
        ([(-hx, s1, hz), (hx, s1, hz), (hx, hy, hz), (-hx, hy, hz)]),
        ([(-hx, s0, hz), (-sx, s0, hz), (-sx, s1, hz), (-hx, s1, hz)]),
        ([(sx, s0, hz), (hx, s0, hz), (hx, s1, hz), (sx, s1, hz)]),
    ]
    for k, c in enumerate(back):
        quads[f"back{k}"] = (c, (0, 0, -1))
    for name, (corners, n) in quads.items():
        p = os.path.join(d, f"room_{name}.obj")
        quad_obj(p, corners, n)
        objs.append(mesh(p, rough()))
    lp = os.path.join(d, "exterior_light.obj")
    lz = hz + 1.0
    quad_obj(lp, [(-1, 2, lz), (-1, 4, lz), (1, 4, lz), (1, 2, lz)], (0, 0, -1))
    objs.append(mesh(lp, diffuse((0, 0, 0)), area_light=(200, 200, 200)))
    cfg = config_json(width, height, spp, depth, accel=accel, threads=threads, integrator=integrator)
    return write_scene(d, cfg, camera((0, 2.0, -4.6), (0, 1.2, 2.0), 60), objs, "slit_room")
