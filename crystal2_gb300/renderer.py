"""Python mirror of the reference's render driver and integrator plug-in surface.

``RayTracer(config, scene)`` follows ``RayTracer`` (src/Core/RayTracer.cpp:11-43): it loads the
two JSON files, builds the scene, camera and integrator, renders into a frame buffer and writes
``result.hdr``.  ``Integrator.load`` mirrors the string factory ``Integrator::LoadIntegrator``
(src/Integrators/Integrator.cpp:14-47): "PathTracer" and "DirectLight" map to the GPU kernels,
anything else raises ``ValueError`` like the reference's ``std::invalid_argument``.
Every computation happens in ``libc2g.so`` on the GPU; nothing here computes pixels.
"""
from __future__ import annotations

import ctypes as C
import json
import os
import struct

import numpy as np

from . import _native as N


class Context:
    """Owns one ``c2g_ctx`` (device memory, stream, loaded scene)."""

    def __init__(self, device: int = 0, mem_limit_bytes: int = 0, verbose: bool = False):
        self._lib = N.load_library()
        self._h = C.c_void_p()
        opts = N.DeviceOpts(device, mem_limit_bytes, 1 if verbose else 0)
        rc = self._lib.c2g_create(C.byref(self._h), C.byref(opts))
        if rc != N.C2G_OK:
            msg = self._lib.c2g_last_error(self._h).decode() if self._h else "create failed"
            if self._h:
                self._lib.c2g_destroy(self._h)
                self._h = C.c_void_p()
            raise N.C2GError(rc, msg)
        self.host_only = device < 0

    @property
    def handle(self):
        return self._h

    def check(self, rc: int) -> None:
        if rc != N.C2G_OK:
            raise N.C2GError(rc, self._lib.c2g_last_error(self._h).decode())

    def close(self) -> None:
        if self._h:
            self._lib.c2g_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- scene
    def register_image(self, path: str, rgb8: np.ndarray) -> None:
        """Decoded (height, width, 3) uint8 pixels used for a texture or skybox file path."""
        a = np.ascontiguousarray(rgb8, np.uint8)
        self.check(self._lib.c2g_register_image(self._h, path.encode(), a.shape[1], a.shape[0],
                                                a.ctypes.data_as(C.POINTER(C.c_ubyte))))

    def load(self, config_path: str, scene_path: str, tree: int = N.TREE_SAH) -> None:
        self.check(self._lib.c2g_load_json(self._h, config_path.encode(), scene_path.encode(), tree))

    def load_text(self, config_json: str, scene_json: str, tree: int = N.TREE_SAH) -> None:
        self.check(self._lib.c2g_load_json_text(self._h, config_json.encode(), scene_json.encode(), tree))

    def build_tree(self, tree: int) -> None:
        self.check(self._lib.c2g_bvh_build(self._h, tree))

    def render_params(self) -> N.RenderParams:
        p = N.RenderParams()
        self.check(self._lib.c2g_get_render_params(self._h, C.byref(p)))
        return p

    def num_objects(self) -> int:
        return self._lib.c2g_num_objects(self._h)

    def num_lights(self) -> int:
        return self._lib.c2g_num_lights(self._h)

    def bvh_order(self) -> np.ndarray:
        n = self.num_objects()
        out = np.zeros(n, np.int32)
        m = self._lib.c2g_bvh_order(self._h, N.iptr(out), n)
        if m < 0:
            self.check(-m if m < 0 else m)
        return out

    def bvh_nodes(self):
        tot = self._lib.c2g_bvh_nodes(self._h, None, None, None, 0)
        if tot < 0:
            self.check(-tot)
        b = np.zeros((tot, 6), np.float32)
        a = np.zeros((tot, 2), np.int32)
        ax = np.zeros(tot, np.int32)
        self._lib.c2g_bvh_nodes(self._h, N.fptr(b), N.iptr(a), N.iptr(ax), tot)
        return b, a, ax

    # ---- rendering
    def render(self, params: N.RenderParams, stream: int | None = None) -> None:
        self.check(self._lib.c2g_render(self._h, C.byref(params), C.c_void_p(stream) if stream else None))

    def film_clear(self) -> None:
        self.check(self._lib.c2g_film_clear(self._h, None))

    def film(self):
        p = self.render_params()
        s = np.zeros((p.height, p.width, 3), np.float32)
        w = np.zeros((p.height, p.width), np.float32)
        self.check(self._lib.c2g_film_download(self._h, N.fptr(s), N.fptr(w)))
        return s, w

    def film_m2(self) -> np.ndarray:
        p = self.render_params()
        m = np.zeros((p.height, p.width, 3), np.float32)
        self.check(self._lib.c2g_film_download_m2(self._h, N.fptr(m)))
        return m

    def image(self) -> np.ndarray:
        p = self.render_params()
        img = np.zeros((p.height, p.width, 3), np.float32)
        self.check(self._lib.c2g_film_image(self._h, N.fptr(img)))
        return img

    def image_rgb8(self, gamma: float = 1 / 2.2) -> np.ndarray:
        """GetImageDataRGB8: (height, width, 3) uint8, rows flipped like image()."""
        p = self.render_params()
        out = np.zeros((p.height, p.width, 3), np.uint8)
        self.check(self._lib.c2g_film_rgb8(self._h, float(gamma), out.ctypes.data_as(C.POINTER(C.c_ubyte))))
        return out

    def write_hdr(self, path: str) -> None:
        """Radiance .hdr of the film image (what the reference writes as result.hdr)."""
        self.check(self._lib.c2g_film_write_hdr(self._h, path.encode()))

    def stats(self) -> N.Stats:
        s = N.Stats()
        self.check(self._lib.c2g_get_stats(self._h, C.byref(s)))
        return s

    def set_counting(self, flags: int) -> None:
        """``native.COUNT_TRAVERSAL`` | ``native.COUNT_TIMING`` (0 = off)."""
        self.check(self._lib.c2g_set_counting(self._h, int(flags)))

    def set_traversal(self, width: int) -> None:
        """SAH traversal variant: 2 (binary nodes) or 4 (four-wide nodes, default)."""
        self.check(self._lib.c2g_set_traversal(self._h, int(width)))

    def set_trace_block(self, threads: int) -> None:
        """Threads per block of the traversal kernels: 64, 128 (default) or 256."""
        self.check(self._lib.c2g_set_trace_block(self._h, int(threads)))

    # ---- ray queries
    def trace_rays(self, o: np.ndarray, d: np.ndarray, any_hit: bool = False, tmin=None, tmax=None, ignore=None):
        o = np.ascontiguousarray(o, np.float32)
        d = np.ascontiguousarray(d, np.float32)
        n = o.shape[0]
        obj = np.zeros(n, np.int32)
        t = None if any_hit else np.zeros(n, np.float32)
        tmin = None if tmin is None else np.ascontiguousarray(tmin, np.float32)
        tmax = None if tmax is None else np.ascontiguousarray(tmax, np.float32)
        ignore = None if ignore is None else np.ascontiguousarray(ignore, np.int32)
        self.check(self._lib.c2g_trace_rays(self._h, n, N.fptr(o), N.fptr(d), N.fptr(tmin), N.fptr(tmax),
                                            N.iptr(ignore), 1 if any_hit else 0, N.iptr(obj), N.fptr(t)))
        return (obj.astype(bool) if any_hit else (obj, t))

    def halton(self, width, height, px, py, sample, ndim) -> np.ndarray:
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        sample = np.ascontiguousarray(sample, np.int32)
        out = np.zeros((px.shape[0], ndim), np.float32)
        self.check(self._lib.c2g_halton(self._h, width, height, px.shape[0], N.iptr(px), N.iptr(py), N.iptr(sample), ndim, N.fptr(out)))
        return out

    def sampler_values(self, px, py, sample, dim: int, two_d: bool = True) -> np.ndarray:
        """Draws of the scene's sampler at flat dimension ``dim``: (n, 2) pairs or (n,) values."""
        px = np.ascontiguousarray(px, np.int32)
        py = np.ascontiguousarray(py, np.int32)
        sample = np.ascontiguousarray(sample, np.int32)
        out = np.zeros((px.shape[0], 2) if two_d else (px.shape[0],), np.float32)
        self.check(self._lib.c2g_sampler_values(self._h, px.shape[0], N.iptr(px), N.iptr(py), N.iptr(sample), int(dim),
                                                1 if two_d else 0, N.fptr(out)))
        return out

    def camera_rays(self, pos2: np.ndarray):
        pos2 = np.ascontiguousarray(pos2, np.float32)
        n = pos2.shape[0]
        o = np.zeros((n, 3), np.float32)
        d = np.zeros((n, 3), np.float32)
        self.check(self._lib.c2g_camera_rays(self._h, n, N.fptr(pos2), N.fptr(o), N.fptr(d)))
        return o, d

    # ---- learned guiding proposal (GuidedPathTracer)
    def guide_reset(self, box_lo, box_hi, seed: int = 0) -> None:
        lo = np.ascontiguousarray(box_lo, np.float32)
        hi = np.ascontiguousarray(box_hi, np.float32)
        self.check(self._lib.c2g_guide_reset(self._h, N.fptr(lo), N.fptr(hi), int(seed)))

    def guide_params(self) -> np.ndarray:
        p = np.zeros(N.GUIDE_PARAMS, np.float32)
        self.check(self._lib.c2g_guide_get_params(self._h, N.fptr(p)))
        return p

    def guide_set_params(self, params: np.ndarray) -> None:
        p = np.ascontiguousarray(params, np.float32)
        assert p.size == N.GUIDE_PARAMS
        self.check(self._lib.c2g_guide_set_params(self._h, N.fptr(p)))

    def guide_eval(self, xnw: np.ndarray) -> np.ndarray:
        """Raw outputs (n, 40) for inputs (n, 9) = position, normal, outgoing direction."""
        x = np.ascontiguousarray(xnw, np.float32).reshape(-1, 9)
        out = np.zeros((x.shape[0], N.GUIDE_OUTPUTS), np.float32)
        self.check(self._lib.c2g_guide_eval(self._h, x.shape[0], N.fptr(x), N.fptr(out)))
        return out

    def guide_gradient(self, samples: np.ndarray):
        """(grad, loss) of sum w * -log q_mix(wi) for samples (n, 14) = x, n, wo, wi, w, p_bsdf."""
        s = np.ascontiguousarray(samples, np.float32).reshape(-1, 14)
        g = np.zeros(N.GUIDE_PARAMS, np.float32)
        loss = C.c_double(0.0)
        self.check(self._lib.c2g_guide_gradient(self._h, s.shape[0], N.fptr(s), N.fptr(g), C.byref(loss)))
        return g, loss.value

    def guide_levels(self, levels: int) -> None:
        """Bounce levels (from the camera hit) served by the guide; 0 = all."""
        self.check(self._lib.c2g_guide_levels(self._h, int(levels)))

    def guide_stats(self):
        """(loss, records, steps) of the last guided training step."""
        loss, rec, steps = C.c_double(0.0), C.c_int(0), C.c_int(0)
        self.check(self._lib.c2g_guide_stats(self._h, C.byref(loss), C.byref(rec), C.byref(steps)))
        return loss.value, rec.value, steps.value

    def guide_batch(self, records_per_wave: int = 1 << 18, windows: int = 4) -> None:
        """Recorded vertices per guided wave and the minibatch windows its Adam steps take in turn."""
        self.check(self._lib.c2g_guide_batch(self._h, int(records_per_wave), int(windows)))

    def guide_regularize(self, kappa_max: float = 500.0, weight_clamp: float = 20.0, decay_steps: float = 0.0) -> None:
        """vMF concentration cap, training-weight clamp (multiple of the mean weight) and learning-rate
        decay (lr / (1 + step / decay_steps); 0 = constant)."""
        self.check(self._lib.c2g_guide_regularize(self._h, float(kappa_max), float(weight_clamp), float(decay_steps)))

    def guide_config(self, learning_rate: float = 2e-3, bsdf_fraction: float = 0.5, warmup_waves: int = 2,
                     train_steps: int = 1) -> None:
        self.check(self._lib.c2g_guide_config(self._h, float(learning_rate), float(bsdf_fraction), int(warmup_waves),
                                              int(train_steps)))


class Batch:
    """Many jobs (contexts with loaded scenes + render parameters) rendered together on one GPU:
    one graph launch with device-side wave loops per job, or per-job graphs on concurrent streams
    (c2g_batch_* in include/c2g.h)."""

    def __init__(self, device: int = 0):
        self._lib = N.load_library()
        h = C.c_void_p()
        rc = self._lib.c2g_batch_create(C.byref(h), device)
        if rc != N.C2G_OK:
            raise N.C2GError(rc, "c2g_batch_create failed")
        self._h = h
        self.jobs: list = []

    def _raise(self, rc: int):
        raise N.C2GError(rc, (self._lib.c2g_batch_last_error(self._h) or b"").decode())

    def add(self, ctx: "Context", params: N.RenderParams) -> int:
        """Add a job; returns its index.  The context must outlive the batch."""
        idx = C.c_int(-1)
        rc = self._lib.c2g_batch_add(self._h, ctx.handle, C.byref(params), C.byref(idx))
        if rc:
            self._raise(rc)
        self.jobs.append(ctx)
        return idx.value

    def tune(self, wave_paths: int, streams: int) -> None:
        rc = self._lib.c2g_batch_tune(self._h, int(wave_paths), int(streams))
        if rc:
            self._raise(rc)

    def autotune(self, wave_paths=(1 << 18, 1 << 19, 1 << 20, 1 << 21), streams=(1, 2, 4, 8), trial_spp: int = 4) -> float:
        wp = np.ascontiguousarray(wave_paths, np.int32)
        sn = np.ascontiguousarray(streams, np.int32)
        best = C.c_double(0.0)
        rc = self._lib.c2g_batch_autotune(self._h, N.iptr(wp), wp.size, N.iptr(sn), sn.size, int(trial_spp), C.byref(best))
        if rc:
            self._raise(rc)
        return best.value

    def set_lanes(self, lanes: int) -> None:
        """One-launch mode: job chains side by side (0 = every job on its own)."""
        rc = self._lib.c2g_batch_set_lanes(self._h, int(lanes))
        if rc:
            self._raise(rc)

    def set_trace(self, traversal: int, trace_block: int) -> None:
        rc = self._lib.c2g_batch_set_trace(self._h, int(traversal), int(trace_block))
        if rc:
            self._raise(rc)

    def search(self, wave_paths=(1 << 19, 1 << 20, 1 << 21, 1 << 22), streams=(0, 8), traversal=(4, 2),
               trace_block=(128, 64, 256), trial_spp: int = 4) -> float:
        """Coordinate search over wave size, mode (0 = one graph launch), traversal variant and the
        traversal kernels' block size; returns the best trial rate (Mpaths/s)."""
        arrs = [np.ascontiguousarray(v, np.int32) for v in (wave_paths, streams, traversal, trace_block)]
        sp = N.BatchSpace(N.iptr(arrs[0]), arrs[0].size, N.iptr(arrs[1]), arrs[1].size, N.iptr(arrs[2]), arrs[2].size,
                          N.iptr(arrs[3]), arrs[3].size)
        best = C.c_double(0.0)
        rc = self._lib.c2g_batch_search(self._h, C.byref(sp), int(trial_spp), C.byref(best))
        if rc:
            self._raise(rc)
        return best.value

    def run(self) -> N.BatchStats:
        st = N.BatchStats()
        rc = self._lib.c2g_batch_run(self._h, C.byref(st))
        if rc:
            self._raise(rc)
        return st

    def latency_ms(self, i: int) -> float:
        v = C.c_double(0.0)
        rc = self._lib.c2g_batch_job_latency(self._h, int(i), C.byref(v))
        if rc:
            self._raise(rc)
        return v.value

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.c2g_batch_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


class Integrator:
    """String factory of the integrators (Integrator::LoadIntegrator)."""

    TYPES = {"PathTracer": N.INTEGRATOR_PATH, "DirectLight": N.INTEGRATOR_DIRECT, "GuidedPathTracer": N.INTEGRATOR_GUIDED}

    def __init__(self, kind: int, depth: int):
        self.kind = kind
        self.depth = depth

    @classmethod
    def load(cls, config: dict) -> "Integrator":
        node = config["Integrator"]
        t = node["Type"]
        if t not in cls.TYPES:
            raise ValueError("Invalid Integrator Type!")
        if node["Sampler"]["Type"] not in ("Halton", "Default", "Stratified"):
            raise ValueError("Invalid Sampler Type!")
        return cls(cls.TYPES[t], int(node["Depth"]))

    def render(self, ctx: Context, sample_begin: int = 0, sample_count: int | None = None, wave_paths: int = 0) -> None:
        """Integrator::Render(Scene*, Camera*, FrameBuffer*) on the context's loaded scene."""
        p = ctx.render_params()
        p.integrator = self.kind
        p.max_depth = self.depth
        p.sample_begin = sample_begin
        p.sample_count = p.spp - sample_begin if sample_count is None else sample_count
        p.wave_paths = wave_paths
        ctx.render(p)


class RayTracer:
    """``RayTracer(config, scene)`` then ``trace()``; ``image()`` is GetImageDataRGB32F."""

    def __init__(self, config_path: str, scene_path: str, device: int = 0, tree: int = N.TREE_SAH):
        with open(config_path) as fh:
            self.config = json.load(fh)
        self.ctx = Context(device)
        self.ctx.load(config_path, scene_path, tree)
        self.integrator = Integrator.load(self.config)

    def trace(self) -> float:
        self.ctx.film_clear()
        self.integrator.render(self.ctx)
        return self.ctx.stats().seconds

    def image(self) -> np.ndarray:
        return self.ctx.image()

    def write_hdr(self, path: str = "result.hdr") -> None:
        self.ctx.write_hdr(path)


def write_hdr(path: str, rgb: np.ndarray) -> None:
    """Radiance .hdr of an (height, width, 3) float image, row 0 written first (no context needed)."""
    a = np.ascontiguousarray(rgb, np.float32)
    rc = N.load_library().c2g_write_hdr(path.encode(), a.shape[1], a.shape[0], N.fptr(a))
    if rc:
        raise N.C2GError(rc, "c2g_write_hdr failed: " + path)

