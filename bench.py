#!/usr/bin/env python3
"""Benchmark: Mpaths/s of the GPU MIS path tracer at 1080p on the many-material scene.

Workload (the configuration the headline metric is quoted on): 400 subdivision-4 icospheres
(2,048,000 triangles) on a jittered 20 x 20 grid over a 40 x 40 ground quad, five material families
(GGX, anisotropic GGX, rough glass, mirror, diffuse), two area quads of radiance 20 plus a point light
of intensity 50; 1920 x 1080, max depth 16, Halton sampler, BVH semantics, SAH tree.  The full
render is 256 spp; one bench step renders `--spp-per-step` samples of every pixel (default 16, i.e.
33.2 M camera paths, one wave of the library's default size), so 16 steps make the full render.

Timing: W untimed warm-up steps, then K steps bracketed by a barrier and device synchronisation,
timed with CUDA events on the stream the kernels run on (max over ranks).  The scene (~200 MB of
BVH/prims) and the wave state (~20 GB) are far larger than the 129 MB L2, so no L2 flush is added.
`e2e` is the same metric through the public C ABI per step: c2g_render (render parameters from the
host) plus the film (rgb sums and weights) read back into pinned host memory (c2g_film_download),
wall-clock timed.

Multi-GPU: the path does not exchange data; `--gpus N` runs N independent replicas (weak scaling),
one process per GPU, rendering the same frame; value = all paths / max time.

The second half of the metric, equal-time relMSE of the guided path tracer against the plain
one, is measured after the timed region on the slit-lit glossy room (`guided_equal_time`): at the
metric's 1920 x 1080 against a 16384-spp plain reference by default (about two minutes; smaller
`--guided-res` / `--guided-ref-spp` for quick runs).

Batched multi-job rendering (64 seeded jobs through replayed CUDA graphs, autotuned wave size and
stream count) is measured last (`batch_run`; `--no-batch` skips it).

`--impl reference` times the reference renderer's own CPU code (compiled from its sources by
oracle/build_ref.py; the oracle port when that library cannot be built) on the host cores, on a
bounded sample of the same workload: rows of the 1080p frame at 1 spp per step.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

WORKLOAD = {
    "workload": "many_material_1080p",
    "scene": "400 icospheres (subdiv 4, 5120 tris each) + 40x40 ground quad, 2,048,002 triangles",
    "materials": "GGX U(0.05,0.8), aniso GGX U(0.05,0.6)^2, glass IOR 1.5 a=0.1, mirror, diffuse U(0.2,0.9)",
    "lights": "2 area quads Le=20 (4 triangle lights) + point light flux 50*4pi",
    "resolution": "1920x1080", "spp_full_render": 256, "max_depth": 16, "sampler": "Halton",
    "tree": "SAH (binned, 16 bins, leaves <= 2), collapsed to four-wide nodes", "accel_semantics": "BVH",
}


def _env_int(k, d):
    try:
        return int(os.environ.get(k, d))
    except ValueError:
        return d


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []
        self.t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.t:
            self.t.join(timeout=2)
        sm, smax, reasons, power = [], [], set(), []
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
                power.append(float(parts[3]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "power_w_max": max(power) if power else None}


def make_scene(out_dir: str, spp: int, scale: float = 1.0):
    from crystal2_gb300 import scenes
    w, h = int(1920 * scale), int(1080 * scale)
    return scenes.many_material(out_dir, width=w, height=h, spp=spp, depth=16, seed=2)


def load_peaks() -> tuple[dict, str]:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as fh:
            return json.load(fh), "of measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0}, "of fallback"


TRAFFIC_FILE = os.path.join(ROOT, "profiles", "traffic_many_material_1080p.md")


def load_traffic(kernel: str) -> dict | None:
    """Measured bytes per ray of `kernel` on this workload from the committed ncu summary: a line
    `per_ray <kernel> dram <bytes> l2 <bytes>` (DRAM read + write, and L2 tag traffic, over the
    launches of one step divided by the rays they traced)."""
    if not os.path.exists(TRAFFIC_FILE):
        return None
    with open(TRAFFIC_FILE) as fh:
        for ln in fh:
            parts = ln.strip().strip("`").split()
            if len(parts) >= 6 and parts[0] == "per_ray" and parts[1] == kernel:
                try:
                    return {"dram": float(parts[3]), "l2": float(parts[5])}
                except ValueError:
                    return None
    return None


def l2_read_peak(device: int) -> float | None:
    """L2 read bandwidth (GB/s) measured by the library's probe: 64 MB read 50 times by every SM
    with L2-only loads (c2g_probe_l2_read); the best of three."""
    import ctypes as C
    from crystal2_gb300 import _native as N
    lib = N.load_library()
    best = None
    for _ in range(3):
        g = C.c_double(0.0)
        if lib.c2g_probe_l2_read(device, 64 << 20, 50, C.byref(g)) == 0:
            best = max(best or 0.0, g.value)
    return best


def cpu_baseline(cfg_dir: str, budget_s: float = 12.0, rows: int | None = None) -> dict:
    """Reference CPU path on a bounded sample: rows of the 1080p frame at 1 spp."""
    from oracle import bindings as B
    cp, sp = make_scene(cfg_dir, spp=1)
    kind = "reference"
    try:
        sc = B.ref_open(cp, sp)
    except Exception:
        kind = "port"
        sc = B.oracle_open(cp, sp)
    threads = min(16, os.cpu_count() or 1)
    W, H = sc.W, sc.H
    if rows is None:
        y0 = H // 2 - 2
        _, _, t = sc.render_region(0, y0, W, y0 + 4, threads=threads) if kind == "reference" else sc.render_region(0, y0, W, y0 + 4, threads=threads)
        rows = int(max(4, min(H, budget_s / max(t, 1e-3) * 4)))
    y0 = max(0, H // 2 - rows // 2)
    y1 = min(H, y0 + rows)
    _, _, t = sc.render_region(0, y0, W, y1, threads=threads)
    paths = W * (y1 - y0)
    return {"value": paths / t / 1e6, "unit": "Mpaths/s", "cores": threads, "kind": kind, "seconds": t,
            "sample": f"rows {y0}..{y1 - 1} of the 1920x1080 frame at 1 spp ({paths} paths), "
                      f"{'reference PathTracingIntegrator::Evaluate compiled from source' if kind == 'reference' else 'oracle port'}, "
                      f"{threads} threads", "rows": rows}


def run_reference(args) -> None:
    rank = _env_int("RANK", 0)
    if rank != 0:
        return
    wdir = tempfile.mkdtemp(prefix="c2g_bench_ref_")
    # calibrate the per-step sample so the whole run stays within a few minutes
    steps, warm = args.steps, args.warmup
    per_step = max(2.0, min(10.0, 150.0 / max(1, steps + warm)))
    cal = cpu_baseline(wdir, budget_s=per_step)
    vals = []
    for i in range(warm + steps):
        r = cpu_baseline(wdir, rows=cal["rows"])
        if i >= warm:
            vals.append(r["value"])
    v = statistics.mean(vals)
    line = {"metric": "Mpaths/s at 1080p (many-material scene, MIS path tracer)", "value": v, "unit": "Mpaths/s",
            "n_gpus": args.gpus, "steps": steps, "warmup": warm, "ms_per_step": 1e3 * cal["rows"] * 1920 / (v * 1e6),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded scene generator)",
            "config": dict(WORKLOAD, parallelism="cpu threads",
                           tree="the reference's own binary BVH, equal-count splits (BVH::Build)",
                           traversal="the reference's stack traversal (BVH::Intersect / IntersectTest)"),
            "impl": "reference",
            "cpu_baseline": {"value": v, "unit": "Mpaths/s", "cores": cal["cores"], "kind": cal["kind"], "sample": cal["sample"]},
            "e2e": {"value": v, "unit": "Mpaths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def replica_rate(t_local: float, paths_local: float, dist=None) -> tuple[float, float]:
    """Whole-job rate of independent replicas: (max time over ranks, Mpaths/s = all ranks' paths
    over that time).  `dist` is torch.distributed with an initialised process group, or None."""
    import torch
    t_max, paths = t_local, paths_local
    if dist is not None:
        tt = torch.tensor([t_local], dtype=torch.float64)
        dist.all_reduce(tt, op=dist.ReduceOp.MAX)
        pp = torch.tensor([paths_local], dtype=torch.float64)
        dist.all_reduce(pp, op=dist.ReduceOp.SUM)
        t_max, paths = float(tt.item()), float(pp.item())
    return t_max, paths / t_max / 1e6


def run_ours(args) -> None:
    import ctypes as C

    import numpy as np
    import torch

    world = _env_int("WORLD_SIZE", 1)
    rank = _env_int("RANK", 0)
    local = _env_int("LOCAL_RANK", 0)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo")
    torch.cuda.set_device(local)
    from crystal2_gb300 import Context
    from crystal2_gb300 import _native as N

    wdir = tempfile.mkdtemp(prefix=f"c2g_bench_{rank}_")
    spp_full = 256
    cp, sp = make_scene(wdir, spp=spp_full, scale=args.scale)
    ctx = Context(local)
    t0 = time.time()
    ctx.set_traversal(args.sah_width)
    ctx.set_trace_block(args.trace_block)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    load_s = time.time() - t0
    p = ctx.render_params()
    sps = args.spp_per_step
    stream = torch.cuda.Stream()
    sh = stream.cuda_stream

    def step(i: int) -> None:
        q = N.RenderParams()
        C.memmove(C.addressof(q), C.addressof(p), C.sizeof(p))
        q.sample_begin = (i * sps) % spp_full
        q.sample_count = sps
        q.wave_paths = args.wave_paths
        ctx.render(q, stream=sh)

    for i in range(args.warmup):
        step(i)
    # traversal counters (untimed): rays, nodes and prims per traversal kernel
    # exclusive per-kernel times (untimed): one step with every kernel on one stream
    ctx.set_counting(N.COUNT_TIMING | N.COUNT_SERIAL)
    step(0)
    sst = ctx.stats()
    serial_ms = np.array(sst.kernel_ms[:])
    serial_n = np.array(sst.kernel_count[:])
    ctx.set_counting(N.COUNT_TRAVERSAL)
    step(0)
    cst = ctx.stats()
    counts = {k: (cst.rays[i], cst.nodes[i], cst.prims[i]) for i, k in ((N.K_EXTEND, "extend"), (N.K_SHADOW, "shadow"), (N.K_MIS, "mis"))}
    level_paths = [int(v) for v in cst.level_paths[:]]
    while level_paths and level_paths[-1] == 0:
        level_paths.pop()
    # timed region (per-launch CUDA events on for the roofline)
    ctx.set_counting(N.COUNT_TIMING)
    clocks = ClockSampler(local)
    if dist:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    ev0 = torch.cuda.Event(enable_timing=True)
    ev1 = torch.cuda.Event(enable_timing=True)
    kernel_ms = np.zeros(N.K_KINDS)
    kernel_n = np.zeros(N.K_KINDS)
    level_ms = np.zeros(N.LEVELS)
    launches = 0
    ev0.record(stream)
    for i in range(args.steps):
        step(args.warmup + i)
        st = ctx.stats()
        kernel_ms += np.array(st.kernel_ms[:])
        kernel_n += np.array(st.kernel_count[:])
        level_ms += np.array(st.level_ms[:])
        launches += st.kernel_launches
    ev1.record(stream)
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    clk = clocks.stop()
    ms = ev0.elapsed_time(ev1)
    ctx.set_counting(0)
    t_local = ms / 1e3
    paths_rank = p.width * p.height * sps * args.steps
    t_max, value = replica_rate(t_local, paths_rank, dist)
    # end to end through the C ABI with host buffers
    # the film read back into pinned host memory (page-locked, as an application streaming frames would)
    film = torch.zeros((p.height, p.width, 3), dtype=torch.float32, pin_memory=True).numpy()
    wgt = torch.zeros((p.height, p.width), dtype=torch.float32, pin_memory=True).numpy()
    e2e_steps = max(2, min(args.steps, 4))
    torch.cuda.synchronize()
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for i in range(e2e_steps):
        q = N.RenderParams()
        C.memmove(C.addressof(q), C.addressof(p), C.sizeof(p))
        q.sample_begin = (i * sps) % spp_full
        q.sample_count = sps
        q.wave_paths = args.wave_paths
        ctx.render(q)
        ctx.check(ctx._lib.c2g_film_download(ctx.handle, N.fptr(film), N.fptr(wgt)))
    e2e_t, e2e = replica_rate(time.perf_counter() - t0, paths_rank / args.steps * e2e_steps, dist)
    # roofline of the dominant kernel: the traversal kernel with the most exclusive device time (the
    # serial step above); the timed region runs kernels of a level side by side on three streams,
    # so there a kernel's event-timed duration includes the time it shares the GPU
    peaks, peak_src = load_peaks()
    names = N.KERNEL_NAMES
    roof = None
    trav = {N.K_EXTEND: "extend", N.K_SHADOW: "shadow", N.K_MIS: "mis"}
    top_trav = max(trav, key=lambda k: serial_ms[k])
    rays, nodes, prims = counts[trav[top_trav]]
    # algorithmic bytes: 32 B ray + 8 B hit + 32 B per node visited + 36 B per triangle tested
    alg_bytes_per_step = 40.0 * rays + 32.0 * nodes + 36.0 * prims
    launches_per_step = kernel_n[top_trav] / args.steps
    avg_launch_s = kernel_ms[top_trav] / 1e3 / max(1, kernel_n[top_trav])
    bytes_per_launch = alg_bytes_per_step / max(1, launches_per_step)
    achieved = bytes_per_launch / max(avg_launch_s, 1e-12) / 1e9
    peak = float(peaks.get("hbm_gbs", 6800.0))
    rays_per_launch = rays / max(1, launches_per_step)
    measured = load_traffic(names[top_trav])
    traffic = None if measured is None else measured["dram"] * rays_per_launch
    iso_s = serial_ms[top_trav] / 1e3 / max(1, serial_n[top_trav])
    roof = {"kernel": names[top_trav], "bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
            "frac": achieved / peak, "peak_source": peak_src, "traffic": traffic,
            "alg_bytes_per_launch": bytes_per_launch, "avg_launch_ms": avg_launch_s * 1e3,
            "duration_note": "CUDA events on the kernel's stream inside the timed region, where the MIS rays and "
                             "the next level's extension run beside it on the other streams",
            "exclusive": {"avg_launch_ms": iso_s * 1e3, "achieved": bytes_per_launch / max(iso_s, 1e-12) / 1e9,
                          "frac": bytes_per_launch / max(iso_s, 1e-12) / 1e9 / peak,
                          "how": "an untimed step with every kernel on one stream (C2G_COUNT_SERIAL)"},
            "per_ray": {"nodes": nodes / max(1, rays), "prims": prims / max(1, rays)}}
    # the roof the traversal actually meets: L2 (the scene's nodes and triangles are re-read by
    # every ray from L2), against an L2 read peak measured on this GPU
    l2_peak = l2_read_peak(local)
    if measured is not None and l2_peak:
        l2_bytes = measured["l2"] * rays_per_launch
        l2_ach = l2_bytes / max(avg_launch_s, 1e-12) / 1e9
        roof["l2"] = {"achieved": l2_ach, "peak": l2_peak, "unit": "GB/s", "frac": l2_ach / l2_peak,
                      "exclusive_frac": l2_bytes / max(iso_s, 1e-12) / 1e9 / l2_peak,
                      "bytes_per_launch": l2_bytes, "dram_frac": traffic / max(avg_launch_s, 1e-12) / 1e9 / peak,
                      "peak_source": "measured: c2g_probe_l2_read (64 MB, 50 reads, L2-only loads, every SM)",
                      "traffic_source": os.path.relpath(TRAFFIC_FILE, ROOT)}
    elif l2_peak:
        roof["l2"] = {"peak": l2_peak, "unit": "GB/s", "achieved": None, "frac": None,
                      "peak_source": "measured: c2g_probe_l2_read (64 MB, 50 reads, L2-only loads, every SM)"}
    # kernel shares of exclusive device time (the serial step; the ncu launch list serialises too)
    share = {names[k]: float(serial_ms[k] / max(1e-9, serial_ms.sum())) for k in range(N.K_KINDS) if serial_n[k] > 0}
    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        try:
            cpu = cpu_baseline(tempfile.mkdtemp(prefix="c2g_cpu_"), budget_s=args.cpu_seconds)
            cpu = {k: cpu[k] for k in ("value", "unit", "cores", "kind", "sample")}
        except Exception as e:  # the baseline is reported, never required
            cpu = {"value": None, "unit": "Mpaths/s", "cores": 0, "kind": "unavailable", "sample": str(e)[:200]}
    guided = None
    if rank == 0 and world == 1 and not args.no_guided:
        try:
            guided = guided_equal_time(args)
        except Exception as e:  # reported beside the headline, never required for it
            guided = {"unavailable": str(e)[:200]}
    rays = None
    if rank == 0 and world == 1 and not args.no_rays:
        try:
            rays = ray_microbench(args)
        except Exception as e:  # reported beside the headline, never required for it
            rays = {"unavailable": str(e)[:200]}
    batch = None
    if rank == 0 and world == 1 and not args.no_batch:
        try:
            batch = batch_run(args)
        except Exception as e:  # reported beside the headline, never required for it
            batch = {"unavailable": str(e)[:200]}
    if rank == 0:
        line = {"metric": "Mpaths/s at 1080p (many-material scene, MIS path tracer)", "value": value, "unit": "Mpaths/s",
                "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": t_max * 1e3 / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded scene generator; no dataset)",
                "config": dict(WORKLOAD, spp_per_step=sps, paths_per_step=p.width * p.height * sps,
                               parallelism=f"replicas x{world}" if world > 1 else "single GPU",
                               l2="inputs larger than L2 (scene + wave state >> 129 MB); no flush",
                               scene_load_s=round(load_s, 2), scale=args.scale,
                               traversal=f"{args.sah_width}-wide nodes, while-while with leaf postponing, "
                                         f"{args.trace_block}-thread blocks"),
                "e2e": {"value": e2e, "unit": "Mpaths/s", "h2d_bytes_per_step": C.sizeof(p),
                        "d2h_bytes_per_step": int(p.width * p.height * 16)},
                "gpu_launches": int(launches), "roofline": roof, "kernel_share": share,
                "traversal_per_step": {k: {"rays": v[0], "nodes": v[1], "prims": v[2]} for k, v in counts.items()},
                "levels": {"paths": level_paths, "ms": [round(float(v) / args.steps, 4) for v in level_ms[:len(level_paths)]]},
                "clocks": clk, "cpu_baseline": cpu, "guided_equal_time": guided, "batch": batch, "ray_microbench": rays}
        print(json.dumps(line), flush=True)
    if dist:
        dist.destroy_process_group()


def time_to_error(curve, err):
    """Render time at which a progressive error curve [(seconds, spp, relMSE), ...] first reaches
    err, interpolated linearly between the two waves around it; None if it never does."""
    if curve and curve[0][2] <= err:
        return curve[0][0]
    for (t0_, _, e0), (t1_, _, e1) in zip(curve, curve[1:]):
        if e1 <= err:  # here e0 > err >= e1
            return t0_ + (t1_ - t0_) * (e0 - err) / (e0 - e1)
    return None


def time_ratio_curve(plain, guided, points=(2.0, 4.0, 6.0, 8.0, 10.0, 15.0, 20.0)):
    """At each point t of plain's curve (its last wave ending by t): the time the guided curve needs
    to reach the error plain had then, over plain's time."""
    out = []
    for t in points:
        if not plain or t > plain[-1][0]:
            break
        before = [p for p in plain if p[0] <= t]
        if not before:
            continue
        t_p, spp_p, err_p = before[-1]
        r = time_to_error(guided, err_p)
        out.append({"plain_s": round(t_p, 2), "plain_spp": spp_p, "relMSE": err_p,
                    "time_ratio": None if r is None else round(r / t_p, 3)})
    return out


def guided_equal_time(args) -> dict:
    """Equal-time error of the guided path tracer against the plain one on the slit-lit glossy room.

    Both arms render the same frame progressively in chunks of `--guided-wave` spp (16: the plain
    tracer's fastest wave size on this scene), one wave per chunk (the guided arm takes
    `--guided-train-steps` Adam steps after each wave), for the same
    budget of render time (the c2g_render calls only; the error is evaluated outside the timer).  relMSE = mean((I - R)^2 / (R^2 + 0.01))
    against a plain reference of `--guided-ref-spp` samples from a disjoint sample range.
    Reported: both errors at the budget, the time the guided arm needs to reach the plain arm's
    error (linear interpolation on its error curve), and their ratio (the target is <= 0.5)."""
    import numpy as np
    from crystal2_gb300 import Context, scenes
    from crystal2_gb300 import _native as N

    W, H = (int(v) for v in args.guided_res.split("x"))
    d = tempfile.mkdtemp(prefix="c2g_guided_")
    cp, sp = scenes.slit_room(d, width=W, height=H, spp=64, depth=12, hf_res=512)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    tiles = ((W + 7) // 8) * ((H + 7) // 8) * 64

    def params(integ, s0, n, wave_spp=1):
        q = ctx.render_params()
        q.integrator, q.sample_begin, q.sample_count, q.wave_paths = integ, s0, n, tiles * wave_spp
        return q

    t0 = time.perf_counter()
    ctx.film_clear()
    ctx.render(params(N.INTEGRATOR_PATH, 1 << 24, args.guided_ref_spp, 8))
    ref = ctx.image().astype(np.float64)
    ref_s = time.perf_counter() - t0

    # relMSE = mean((I - R)^2 / (R^2 + 0.01)), evaluated in FP32 with the weights precomputed
    # (outside the timed render calls; it only bounds the benchmark's own run time)
    ref32 = ref.astype(np.float32)
    inv = (1.0 / (ref32 * ref32 + 1e-2)).astype(np.float32)

    def relmse(img):
        d = img.astype(np.float32) - ref32
        return float(np.mean(d * d * inv, dtype=np.float64))

    ws = args.guided_wave

    def progressive(integ, wave_spp):
        ctx.film_clear()
        s0, spent, curve = 0, 0.0, []
        while spent < args.guided_seconds:
            t = time.perf_counter()
            ctx.render(params(integ, s0, wave_spp, wave_spp))
            spent += time.perf_counter() - t
            s0 += wave_spp
            curve.append((spent, s0, relmse(ctx.image())))
        return curve

    ctx.film_clear()
    ctx.render(params(N.INTEGRATOR_PATH, 0, 4))  # first-launch costs out of the way
    # both arms render 8-sample waves (the guided arm trains after every wave)
    plain = progressive(N.INTEGRATOR_PATH, ws)
    ctx.load(cp, sp, tree=N.TREE_SAH)  # a fresh, untrained network
    ctx.guide_config(args.guided_lr, args.guided_bsdf_fraction, args.guided_warmup, args.guided_train_steps)
    ctx.guide_levels(args.guided_levels)
    ctx.guide_batch(args.guided_records, args.guided_windows)
    ctx.guide_regularize(args.guided_kappa, 20.0, args.guided_lr_decay)
    guided = progressive(N.INTEGRATOR_GUIDED, ws)
    target = plain[-1][2]
    reach = time_to_error(guided, target)
    checkpoints = time_ratio_curve(plain, guided)
    loss, records, steps = ctx.guide_stats()
    # one timed wave of each arm (the trained network): device time per kernel kind
    wave_ms = {}
    ctx.set_counting(N.COUNT_TIMING)
    for name, integ in (("plain", N.INTEGRATOR_PATH), ("guided", N.INTEGRATOR_GUIDED)):
        ctx.render(params(integ, 1 << 20, ws, ws))
        st = ctx.stats()
        wave_ms[name] = {"total": round(st.seconds * 1e3, 2),
                         **{N.KERNEL_NAMES[k]: round(st.kernel_ms[k], 2) for k in range(N.K_KINDS) if st.kernel_count[k] > 0}}
    ctx.set_counting(0)
    return {"scene": f"slit_room {W}x{H} (524k-triangle heightfield, GGX a U(0.1,0.3), slit-lit), max depth 12",
            "reference_spp": args.guided_ref_spp, "reference_s": round(ref_s, 2), "budget_s": args.guided_seconds,
            "plain": {"spp": plain[-1][1], "s": round(plain[-1][0], 3), "relMSE": target, "samples_per_wave": ws},
            "guided": {"spp": guided[-1][1], "s": round(guided[-1][0], 3), "relMSE": guided[-1][2],
                       "bsdf_fraction": args.guided_bsdf_fraction, "learning_rate": args.guided_lr,
                       "train_steps_per_wave": args.guided_train_steps, "samples_per_wave": ws,
                       "records_per_wave": args.guided_records, "minibatch_windows": args.guided_windows,
                       "warmup_waves": args.guided_warmup, "kappa_max": args.guided_kappa, "lr_decay_steps": args.guided_lr_decay,
                       "guided_levels": args.guided_levels,
                       "adam_steps": steps, "last_batch": records, "last_loss": round(loss, 4)},
            "time_to_plain_relMSE_s": None if reach is None else round(reach, 3),
            "time_ratio": None if reach is None else round(reach / plain[-1][0], 3),
            "time_ratio_curve": checkpoints,
            "equal_time_relMSE_ratio": round(guided[-1][2] / target, 3),
            "wave_ms": wave_ms, "wave_ms_note": "one wave per arm with per-launch CUDA events; kernels on the "
                                                "side stream overlap, so the kinds can sum past the total"}


def batch_run(args) -> dict:
    """Batched multi-job rendering: `--batch-jobs` seeded jobs (Cornell and many-material variants,
    square resolutions log-uniform in [128, 1024], spp from {16, 64, 256, 1024}, guided or plain)
    rendered together on one GPU.  The library's coordinate search picks, on a 4-spp trial of every
    job, the wave size, the mode (0 = the whole batch as one graph launch with device-side wave
    loops per job; S > 0 = per-job wave graphs on S streams), the traversal variant (two- or
    four-wide nodes) and the traversal kernels' block size."""
    import numpy as np
    from crystal2_gb300 import Batch, Context, scenes
    from crystal2_gb300 import _native as N

    t0 = time.time()
    jobs = scenes.batch_jobs(tempfile.mkdtemp(prefix="c2g_batch_"), n_jobs=args.batch_jobs)
    ctxs = []
    b = Batch(0)
    n_guided = 0
    for cp, sp, spp, guided in jobs:
        c = Context(0)
        c.load(cp, sp, tree=N.TREE_SAH)
        p = c.render_params()
        p.integrator = N.INTEGRATOR_GUIDED if guided else N.INTEGRATOR_PATH
        p.sample_begin, p.sample_count = 0, spp
        c.film_clear()
        b.add(c, p)
        ctxs.append(c)
        n_guided += int(guided)
    load_s = time.time() - t0
    t0 = time.time()
    best = b.search(wave_paths=(1 << 21, 1 << 22, 1 << 23), streams=(0, 8), traversal=(4, 2),
                    trace_block=(128, 64, 256), trial_spp=8)
    tune_s = time.time() - t0
    st = b.run()
    lat = [b.latency_ms(i) for i in range(len(jobs))]
    one = None
    if st.streams != 0:
        # the one-launch mode with the same wave size and traversal, from fresh films and networks
        for c, (_, _, _, guided) in zip(ctxs, jobs):
            c.film_clear()
            if guided:
                c.guide_reset((0.0, 0.0, 0.0), (1.0, 1.0, 1.0), seed=0)
        b.tune(st.wave_paths, 0)
        s1 = b.run()
        one = {"mpaths_per_s": round(s1.mpaths_per_s, 2), "seconds": round(s1.seconds, 3), "graph_launches": s1.graph_launches,
               "latency_p50_ms": round(s1.latency_p50_ms, 2), "latency_p90_ms": round(s1.latency_p90_ms, 2),
               "latency_max_ms": round(s1.latency_max_ms, 2), "latency_mean_ms": round(s1.latency_mean_ms, 2)}
    out = {"jobs": st.jobs, "guided_jobs": n_guided, "paths": st.paths, "seconds": round(st.seconds, 3),
           "mpaths_per_s": round(st.mpaths_per_s, 2), "latency_p50_ms": round(st.latency_p50_ms, 2),
           "latency_p90_ms": round(st.latency_p90_ms, 2), "latency_p99_ms": round(st.latency_p99_ms, 2),
           "latency_max_ms": round(st.latency_max_ms, 2), "latency_mean_ms": round(st.latency_mean_ms, 2),
           "latency_rule": "nearest rank over the jobs' completion times from the batch start",
           "tuned": {"wave_paths": st.wave_paths, "mode": "one graph launch" if st.streams == 0 else f"{st.streams} streams",
                     "traversal": f"{st.traversal}-wide nodes", "trace_block": st.trace_block,
                     "trial_mpaths_per_s": round(best, 2), "tune_s": round(tune_s, 2)},
           "graph_launches": st.graph_launches, "one_launch_mode": one, "scene_load_s": round(load_s, 1),
           "resolutions": [int(c.render_params().width) for c in ctxs],
           "latency_ms": [round(x, 2) for x in lat]}
    b.close()
    for c in ctxs:
        c.close()
    return out


def ray_microbench(args) -> dict:
    """Ray-intersection microbench: 1M-triangle soup (centroids U[0,1]^3, vertices +- 0.005) in the
    SAH tree, 16M rays (8M pinhole primaries of a 4096^2 image of the cube, 8M random origins and
    directions), closest hit and then any hit with tmax ~ U(0, 2 t_closest); device-resident rays
    through c2g_trace_rays_dev, CUDA-event timed over `--steps` launches after 3 warm-up launches."""
    import ctypes as C

    import numpy as np
    import torch
    from crystal2_gb300 import Context, scenes
    from crystal2_gb300 import _native as N

    d = tempfile.mkdtemp(prefix="c2g_rays_")
    cp, sp = scenes.tri_soup(d, n_tris=1 << 20)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    n = args.rays
    o, dd = scenes.microbench_rays(n)
    dev = torch.device("cuda", 0)
    to = torch.from_numpy(o).to(dev)
    td = torch.from_numpy(dd).to(dev)
    obj = torch.empty(n, dtype=torch.int32, device=dev)
    t = torch.empty(n, dtype=torch.float32, device=dev)
    stream = torch.cuda.Stream()
    lib = ctx._lib

    def launch(any_hit, tmin=None, tmax=None):
        p = lambda x: C.c_void_p(x.data_ptr()) if x is not None else None
        rc = lib.c2g_trace_rays_dev(ctx.handle, n, p(to), p(td), p(tmin), p(tmax), None, int(any_hit), p(obj),
                                    None if any_hit else p(t), C.c_void_p(stream.cuda_stream))
        ctx.check(rc)

    def timed(any_hit, tmin=None, tmax=None):
        for _ in range(3):
            launch(any_hit, tmin, tmax)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(stream)
        for _ in range(args.steps):
            launch(any_hit, tmin, tmax)
        e1.record(stream)
        torch.cuda.synchronize()
        return e0.elapsed_time(e1) / 1e3 / args.steps

    s_closest = timed(False)
    tc = t.clone()
    hit = torch.isfinite(tc) & (obj >= 0)
    g = torch.Generator(device="cpu").manual_seed(5)
    u = torch.rand(n, generator=g).to(dev)
    tmax = torch.where(hit, 2.0 * tc * u, torch.full_like(u, 4.0) * u).contiguous()
    tmin = torch.zeros(n, dtype=torch.float32, device=dev)
    s_any = timed(True, tmin, tmax)
    return {"scene": "1M-triangle soup (SAH tree, four-wide nodes)", "rays": n,
            "closest_mrays_per_s": round(n / s_closest / 1e6, 1), "anyhit_mrays_per_s": round(n / s_any / 1e6, 1),
            "closest_hit_fraction": round(float(hit.float().mean().item()), 4)}


def main() -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp-per-step", type=int, default=16)
    ap.add_argument("--scale", type=float, default=1.0, help="film scale (1.0 = 1920x1080)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-guided", action="store_true", help="skip the guided-vs-plain equal-time measurement")
    ap.add_argument("--guided-res", default="1920x1080")
    ap.add_argument("--guided-ref-spp", type=int, default=16384)
    ap.add_argument("--guided-seconds", type=float, default=10.0, help="render time per arm of the guided leg")
    ap.add_argument("--guided-lr", type=float, default=1e-3)
    ap.add_argument("--guided-bsdf-fraction", type=float, default=0.7)
    ap.add_argument("--guided-train-steps", type=int, default=64,
                    help="Adam steps per guided wave (64: no collapse in eight 10 s runs; 128 learned faster but "
                         "collapsed in two of seven)")
    ap.add_argument("--guided-records", type=int, default=1 << 21, help="recorded vertices per guided wave")
    ap.add_argument("--guided-windows", type=int, default=32, help="minibatch windows per guided wave")
    ap.add_argument("--guided-wave", type=int, default=16, help="samples per pixel per wave, both arms (plain's fastest)")
    ap.add_argument("--guided-warmup", type=int, default=1, help="guided waves that only train")
    ap.add_argument("--guided-kappa", type=float, default=200.0, help="vMF concentration cap of the guide mixture")
    ap.add_argument("--guided-lr-decay", type=float, default=2000.0, help="Adam steps over which the learning rate halves (0 = constant)")
    ap.add_argument("--guided-levels", type=int, default=0, help="bounce levels served by the guide (0 = all)")
    ap.add_argument("--no-batch", action="store_true", help="skip the batched multi-job measurement")
    ap.add_argument("--sah-width", type=int, default=4, choices=[2, 4], help="SAH traversal variant")
    ap.add_argument("--trace-block", type=int, default=128, choices=[64, 128, 256], help="traversal kernels' block size")
    ap.add_argument("--wave-paths", type=int, default=0, help="paths per wave (0: the library default, 2^21)")
    ap.add_argument("--batch-jobs", type=int, default=64)
    ap.add_argument("--no-rays", action="store_true", help="skip the ray-intersection microbench")
    ap.add_argument("--rays", type=int, default=1 << 24)
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)
    return 0


if __name__ == "__main__":
    sys.exit(main())
