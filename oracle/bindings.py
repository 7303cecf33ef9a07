"""ctypes bindings of the two checkers: the oracle port (``libc2oracle.so``) and the compiled
reference (``oracle/_ref/libc2ref.so``).

TEST INFRASTRUCTURE ONLY: imported by tests/, ``__graft_entry__.smoke()`` and bench.py's CPU
baseline leg.  Product code never imports this module.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
_F = C.POINTER(C.c_float)
_D = C.POINTER(C.c_double)
_I = C.POINTER(C.c_int)
_L = C.POINTER(C.c_longlong)


def _f(a):
    return None if a is None else a.ctypes.data_as(_F)


def _d(a):
    return None if a is None else a.ctypes.data_as(_D)


def _i(a):
    return None if a is None else a.ctypes.data_as(_I)


class _Scene:
    """Common interface: one loaded (config, scene) pair in a checker library."""

    prefix = ""

    def __init__(self, lib, cfg: str, scn: str):
        self.lib = lib
        err = C.create_string_buffer(1024)
        h = getattr(lib, self.prefix + "open")(cfg.encode(), scn.encode(), err, 1024)
        if not h:
            raise RuntimeError(err.value.decode())
        self.h = C.c_void_p(h)
        with open(cfg) as fh:
            import json
            c = json.load(fh)
        self.W, self.H, self.spp = c["Width"], c["Height"], c["SamplesPerPixel"]

    def close(self):
        if self.h:
            getattr(self.lib, self.prefix + "close")(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def num_objects(self) -> int:
        return getattr(self.lib, self.prefix + "num_objects")(self.h)

    def num_lights(self) -> int:
        return getattr(self.lib, self.prefix + "num_lights")(self.h)

    def camera(self, pos2):
        pos2 = np.ascontiguousarray(pos2, np.float32)
        n = pos2.shape[0]
        o = np.zeros((n, 3), np.float32)
        d = np.zeros((n, 3), np.float32)
        getattr(self.lib, self.prefix + "camera")(self.h, n, _f(pos2), _f(o), _f(d))
        return o, d


class RefScene(_Scene):
    prefix = "ref_"

    def bvh_order(self):
        o = np.zeros(self.num_objects(), np.int32)
        self.lib.ref_bvh_order(self.h, _i(o))
        return o

    def bvh_nodes(self):
        tot = self.lib.ref_bvh_nodes(self.h, None, None, None)
        b = np.zeros((tot, 6), np.float32)
        a = np.zeros((tot, 2), np.int32)
        ax = np.zeros(tot, np.int32)
        self.lib.ref_bvh_nodes(self.h, _f(b), _i(a), _i(ax))
        return b, a, ax

    def intersect(self, o, d, threads=8):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        obj = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        self.lib.ref_intersect(self.h, n, _f(o), _f(d), _i(obj), _f(t), threads)
        return obj, t

    def intersect_test(self, o, d, tmin, tmax, ignore):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        occ = np.zeros(n, np.int32)
        self.lib.ref_intersect_test(self.h, n, _f(o), _f(d), _f(np.ascontiguousarray(tmin, np.float32)),
                                    _f(np.ascontiguousarray(tmax, np.float32)), _i(np.ascontiguousarray(ignore, np.int32)), _i(occ))
        return occ.astype(bool)

    def render_region(self, x0, y0, x1, y1, threads=8):
        w, h = x1 - x0, y1 - y0
        s = np.zeros((h, w, 3))
        q = np.zeros((h, w, 3))
        secs = self.lib.ref_render_region(self.h, threads, x0, y0, x1, y1, _d(s), _d(q))
        return s, q, secs

    def render_region_groups(self, x0, y0, x1, y1, group, threads=8):
        """Per-pixel sums of each run of `group` consecutive samples (planes of independent
        estimates), the sum of squares over all samples, and the wall seconds."""
        w, h = x1 - x0, y1 - y0
        ng = (self.spp + group - 1) // group
        s = np.zeros((ng, h, w, 3))
        q = np.zeros((h, w, 3))
        secs = self.lib.ref_render_region_groups(self.h, threads, x0, y0, x1, y1, group, _d(s), _d(q))
        return s, q, secs

    def intersect_test_mt(self, o, d, tmin, tmax, ignore=None, threads=8):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        if ignore is None:
            ignore = np.full(n, -1, np.int32)
        occ = np.zeros(n, np.int32)
        self.lib.ref_intersect_test_mt(self.h, n, _f(o), _f(d), _f(np.ascontiguousarray(tmin, np.float32)),
                                       _f(np.ascontiguousarray(tmax, np.float32)), _i(np.ascontiguousarray(ignore, np.int32)),
                                       _i(occ), threads)
        return occ.astype(bool)

    def render(self, threads=8):
        s = np.zeros((self.H, self.W, 3), np.float32)
        w = np.zeros((self.H, self.W), np.float32)
        secs = self.lib.ref_render(self.h, threads, _f(s), _f(w))
        return s, w, secs

    def render_samples(self, px, py):
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        out = np.zeros((px.shape[0], self.spp, 3), np.float32)
        self.lib.ref_render_samples(self.h, px.shape[0], _i(px), _i(py), _f(out))
        return out


class OracleScene(_Scene):
    prefix = "orc_"

    def bvh_order(self):
        o = np.zeros(self.num_objects(), np.int32)
        self.lib.orc_bvh_order(self.h, _i(o))
        return o

    def bvh_nodes(self):
        tot = self.lib.orc_bvh_nodes(self.h, None, None, None)
        b = np.zeros((tot, 6), np.float32)
        a = np.zeros((tot, 2), np.int32)
        ax = np.zeros(tot, np.int32)
        self.lib.orc_bvh_nodes(self.h, _f(b), _i(a), _i(ax))
        return b, a, ax

    def intersect(self, o, d):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        obj = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        self.lib.orc_intersect(self.h, n, _f(o), _f(d), _i(obj), _f(t))
        return obj, t

    def intersect_test(self, o, d, tmin, tmax, ignore):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        occ = np.zeros(n, np.int32)
        self.lib.orc_intersect_test(self.h, n, _f(o), _f(d), _f(np.ascontiguousarray(tmin, np.float32)),
                                    _f(np.ascontiguousarray(tmax, np.float32)), _i(np.ascontiguousarray(ignore, np.int32)), _i(occ))
        return occ.astype(bool)

    def render_region(self, x0, y0, x1, y1, s0=0, ns=None, threads=8, seed=0):
        ns = self.spp if ns is None else ns
        w, h = x1 - x0, y1 - y0
        s = np.zeros((h, w, 3))
        q = np.zeros((h, w, 3))
        secs = self.lib.orc_render_region(self.h, threads, x0, y0, x1, y1, s0, ns, C.c_ulonglong(seed), _d(s), _d(q))
        return s, q, secs

    def set_counter_sampler(self, on: bool) -> None:
        """Draw Default / Stratified values per (pixel, sample, dim) as the library does."""
        self.lib.orc_set_counter_sampler(self.h, 1 if on else 0)

    def render_frame(self, threads=8):
        """(float sum (H, W, 3), float weight (H, W)) accumulated like the reference's FrameBuffer."""
        rgbw = np.zeros((self.H, self.W, 4), np.float32)
        self.lib.orc_render_frame(self.h, threads, _f(rgbw))
        return rgbw[..., :3].copy(), rgbw[..., 3].copy()

    def render_samples(self, px, py, spp=None, seed=0):
        spp = self.spp if spp is None else spp
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        out = np.zeros((px.shape[0], spp, 3), np.float32)
        self.lib.orc_render_samples(self.h, px.shape[0], _i(px), _i(py), spp, C.c_ulonglong(seed), _f(out))
        return out


def _declare(lib, prefix: str) -> None:
    vp = C.c_void_p
    getattr(lib, prefix + "open").restype = vp
    getattr(lib, prefix + "open").argtypes = [C.c_char_p, C.c_char_p, C.c_char_p, C.c_int]
    for name in ("close",):
        getattr(lib, prefix + name).argtypes = [vp]
    for name in ("num_objects", "num_lights"):
        getattr(lib, prefix + name).argtypes = [vp]
        getattr(lib, prefix + name).restype = C.c_int
    getattr(lib, prefix + "camera").argtypes = [vp, C.c_int, _F, _F, _F]
    getattr(lib, prefix + "bvh_order").argtypes = [vp, _I]
    getattr(lib, prefix + "bvh_nodes").argtypes = [vp, _F, _I, _I]
    getattr(lib, prefix + "bvh_nodes").restype = C.c_int
    getattr(lib, prefix + "halton").argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _I, _I, _I, C.c_int, _F] if prefix == "ref_" else \
        [C.c_int, C.c_int, C.c_int, _I, _I, _I, C.c_int, _F]
    getattr(lib, prefix + "intersect_test").argtypes = [vp, C.c_int, _F, _F, _F, _F, _I, _I]


_ref_lib = None
_orc_lib = None


def ref_library():
    """The compiled reference (built on demand from the scratch copy or the reference tree)."""
    global _ref_lib
    if _ref_lib is None:
        from . import build_ref
        path = build_ref.build()
        lib = C.CDLL(path)
        _declare(lib, "ref_")
        lib.ref_intersect.argtypes = [C.c_void_p, C.c_int, _F, _F, _I, _F, C.c_int]
        lib.ref_render.argtypes = [C.c_void_p, C.c_int, _F, _F]
        lib.ref_render.restype = C.c_double
        lib.ref_render_region.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D, _D]
        lib.ref_render_region.restype = C.c_double
        lib.ref_render_region_groups.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, _D, _D]
        lib.ref_render_region_groups.restype = C.c_double
        lib.ref_intersect_test_mt.argtypes = [C.c_void_p, C.c_int, _F, _F, _F, _F, _I, _I, C.c_int]
        lib.ref_render_samples.argtypes = [C.c_void_p, C.c_int, _I, _I, _F]
        lib.ref_write_hdr.argtypes = [C.c_char_p, C.c_int, C.c_int, _F]
        lib.ref_write_hdr.restype = C.c_int
        lib.ref_halton_index.argtypes = [C.c_int, C.c_int, C.c_int, C.c_int, _I, _I, _I, _L]
        lib.ref_bsdf.argtypes = [C.c_char_p, C.c_int, _F, C.c_int, _F, _F, _F, C.c_int, _F, _F, _F, _F, _F, _I]
        lib.ref_bsdf.restype = C.c_int
        lib.ref_light_info.argtypes = [C.c_void_p, C.c_int, _I, _I, _F]
        lib.ref_light_sample.argtypes = [C.c_void_p, C.c_int, C.c_int, _F, _F, _F, _F, _F, _F]
        lib.ref_light_pdf.argtypes = [C.c_void_p, C.c_int, C.c_int, _F, _F, _F, _F]
        _ref_lib = lib
    return _ref_lib


def oracle_library():
    """The oracle port (built on demand)."""
    global _orc_lib
    if _orc_lib is None:
        from . import build_oracle
        lib = C.CDLL(build_oracle.build())
        _declare(lib, "orc_")
        lib.orc_intersect.argtypes = [C.c_void_p, C.c_int, _F, _F, _I, _F]
        lib.orc_render_region.argtypes = [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int,
                                          C.c_ulonglong, _D, _D]
        lib.orc_render_region.restype = C.c_double
        lib.orc_render_samples.argtypes = [C.c_void_p, C.c_int, _I, _I, C.c_int, C.c_ulonglong, _F]
        lib.orc_render_frame.argtypes = [C.c_void_p, C.c_int, _F]
        lib.orc_set_counter_sampler.argtypes = [C.c_void_p, C.c_int]
        lib.orc_bsdf.argtypes = [C.c_char_p, _F, C.c_int, _F, C.c_int, _F, _F, _F, C.c_int, _F, _F, _F, _F, _F, _I]
        lib.orc_bsdf.restype = C.c_int
        _orc_lib = lib
    return _orc_lib


def ref_available() -> bool:
    try:
        ref_library()
        return True
    except Exception:
        return False


def ref_open(cfg: str, scn: str) -> RefScene:
    return RefScene(ref_library(), cfg, scn)


def oracle_open(cfg: str, scn: str) -> OracleScene:
    return OracleScene(oracle_library(), cfg, scn)


def oracle_halton(W, H, px, py, sample, ndim):
    lib = oracle_library()
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    sample = np.ascontiguousarray(sample, np.int32)
    out = np.zeros((px.shape[0], ndim), np.float32)
    lib.orc_halton(W, H, px.shape[0], _i(px), _i(py), _i(sample), ndim, _f(out))
    return out


def ref_halton(W, H, spp, px, py, sample, ndim):
    lib = ref_library()
    px = np.ascontiguousarray(px, np.int32)
    py = np.ascontiguousarray(py, np.int32)
    sample = np.ascontiguousarray(sample, np.int32)
    out = np.zeros((px.shape[0], ndim), np.float32)
    lib.ref_halton(W, H, spp, px.shape[0], _i(px), _i(py), _i(sample), ndim, _f(out))
    return out


BSDF_KINDS = ["Diffuse", "Mirror", "GlassRough", "GlassSmooth", "MicroGGX", "MicroBeckmann", "PlasticGGX", "PlasticBeckmann"]


def material_json(kind: str, params) -> str:
    """The reference's material JSON for an oracle BSDF kind + params (color3, ks3, ax, ay, ior)."""
    import json
    c = [float(x) for x in params[0:3]]
    ks = [float(x) for x in params[3:6]]
    ax, ay, ior = float(params[6]), float(params[7]), float(params[8])
    if kind == "Diffuse":
        m = {"Type": "Diffuse", "Color": c}
    elif kind == "Mirror":
        m = {"Type": "Mirror", "Color": c}
    elif kind in ("GlassRough", "GlassSmooth"):
        m = {"Type": "Glass", "Color": c, "Roughness": [ax, ay], "IOR": ior}
    elif kind.startswith("Micro"):
        m = {"Type": "Micro", "Color": c, "Roughness": [ax, ay], "IOR": ior, "NDF": "GGX" if kind.endswith("GGX") else "Beckmann"}
    elif kind == "OrenNayar":
        m = {"Type": "OrenNayar", "Color": c, "Sigma": ior}
    elif kind == "Phong":
        m = {"Type": "Phong", "Color": c, "K": int(ior)}
    else:
        m = {"Type": "Plastic", "Kd": c, "Ks": ks, "Roughness": [ax, ay], "NDF": "GGX" if kind.endswith("GGX") else "Beckmann"}
    return json.dumps(m)


def bsdf_eval(which: str, kind: str, params, front: int, frame, wo, wi, u3, flags: int):
    """Run the BSDF harness of the oracle ('orc') or the reference ('ref')."""
    n = wo.shape[0]
    fe = np.zeros((n, 3), np.float32)
    pe = np.zeros(n, np.float32)
    fs = np.zeros((n, 3), np.float32)
    ws = np.zeros((n, 3), np.float32)
    ps = np.zeros(n, np.float32)
    ts = np.zeros(n, np.int32)
    frame = np.ascontiguousarray(frame, np.float32)
    wo = np.ascontiguousarray(wo, np.float32)
    wi = np.ascontiguousarray(wi, np.float32)
    u3 = np.ascontiguousarray(u3, np.float32)
    if which == "orc":
        p = np.ascontiguousarray(params, np.float32)
        rc = oracle_library().orc_bsdf(kind.encode(), _f(p), front, _f(frame), n, _f(wo), _f(wi), _f(u3), flags,
                                      _f(fe), _f(pe), _f(fs), _f(ws), _f(ps), _i(ts))
    else:
        rc = ref_library().ref_bsdf(material_json(kind, params).encode(), front, _f(frame), n, _f(wo), _f(wi), _f(u3), flags,
                                    _f(fe), _f(pe), _f(fs), _f(ws), _f(ps), _i(ts))
    if rc < 0:
        raise RuntimeError("bsdf harness failed")
    return fe, pe, fs, ws, ps, ts


def ref_write_hdr(path: str, rgb: np.ndarray) -> None:
    """The reference's stbi_write_hdr on an (h, w, 3) float image (row 0 written first)."""
    a = np.ascontiguousarray(rgb, np.float32)
    if not ref_library().ref_write_hdr(path.encode(), a.shape[1], a.shape[0], _f(a)):
        raise OSError("stbi_write_hdr failed: " + path)
