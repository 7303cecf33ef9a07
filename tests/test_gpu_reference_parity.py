"""GPU parity against the reference renderer itself, on the configurations the numbers are quoted on.

The checker is oracle/_ref/libc2ref.so: the reference's own translation units compiled from its
sources (oracle/build_ref.py), driven through oracle/ref_harness.cpp, which only wires inputs to
the reference's classes (Scene::Intersect / IntersectTest, PathTracingIntegrator::Evaluate under
SamplerIntegrator::Render's pixel/sample loop).  The GPU side is libc2g.so through its C ABI.

* Ray-intersection microbench scene (1M-triangle soup, rays of the 16M-ray microbench): closest-hit
  object ids equal the reference's BVH::Intersect (src/Accelerators/BVH.cpp:56-108) except at
  near-ties, which an FP64 brute-force solve classifies; t within 1e-5 relative of FP64; any-hit
  equal to BVH::IntersectTest (BVH.cpp:110-154) at the microbench's random tmax.
* Cornell box at its full configuration (256^2, 64 spp, depth 8): the relMSE of 64-spp images
  against a 16384-spp converged plain GPU render agrees with the reference CPU's within 2%, and
  per-pixel means agree within 3 standard errors.
* Many-material scene at 1920 x 1080, 16 spp, depth 16: a band of rows, per-pixel z-test against
  the reference (Halton dimensions >= 100 are a hash on the GPU and an unsynchronised global
  mt19937 in the reference, so that part of the agreement is in distribution only).
* Slit-lit room: the full 512^2 heightfield under BVH semantics, and under Brute semantics (exact
  shadow interval, the semantics the guided measurement uses) with a 16^2 heightfield, which keeps
  the reference's linear-scan accelerator (src/Accelerators/Brute.cpp:19-55) affordable.  The
  guided estimator is unbiased on the slit room too.

A note on the aarch64 build of the reference: `bsdf.SampleDirection(sampler->Get1D(),
sampler->Get2D(), ...)` (PathTracingIntegrator.cpp:73-74) evaluates its arguments right to left
with x86-64 g++ and left to right with aarch64 g++, so on an Arm host the reference draws the same
estimator with its sampler dimensions assigned differently: agreement there is statistical, which
is what these tests check.
"""
import os

import numpy as np
import pytest

from crystal2_gb300 import Context, scenes
from crystal2_gb300 import _native as N

pytestmark = pytest.mark.gpu

THREADS = max(1, min(16, os.cpu_count() or 1))


@pytest.fixture(scope="module", autouse=True)
def _built():
    from crystal2_gb300 import build
    build.build()


@pytest.fixture(scope="module")
def ref():
    """The reference library (compiled from its sources on this host); skipped where it cannot
    be built (no reference tree and no scratch copy)."""
    from oracle import bindings as B
    from oracle import build_ref
    try:
        build_ref.build()
        B.ref_library()
    except Exception as e:  # pragma: no cover - depends on the host
        pytest.skip(f"reference library unavailable: {e}")
    return B


def _gpu_film(ctx, sample_begin, sample_count, accel=None, wave_paths=0):
    p = ctx.render_params()
    p.sample_begin, p.sample_count, p.wave_paths = sample_begin, sample_count, wave_paths
    if accel is not None:
        p.accel = accel
    ctx.film_clear()
    ctx.render(p)
    s, w = ctx.film()
    return s.astype(np.float64), ctx.film_m2().astype(np.float64)


def _zscores(s_a, q_a, n_a, s_b, q_b, n_b):
    """Per pixel-channel z of the difference of two sample means (sums s, sums of squares q)."""
    ma, mb = s_a / n_a, s_b / n_b
    va = np.maximum(q_a / n_a - ma ** 2, 0) / n_a
    vb = np.maximum(q_b / n_b - mb ** 2, 0) / n_b
    se = np.sqrt(va + vb)
    z = np.where(se > 0, (ma - mb) / np.where(se > 0, se, 1), np.where(ma == mb, 0.0, np.inf))
    return z, ma, mb, va + vb


def _relmse(img, R):
    return float(np.mean((img - R) ** 2 / (R ** 2 + 1e-2)))


# ---- ray-intersection microbench scene ------------------------------------------------------------

def _fp64_hits(o, d, tris):
    """Double-precision ray/triangle solve of one ray against many triangles: t (inf on a miss)."""
    o = np.asarray(o, np.float64)
    d = np.asarray(d, np.float64)
    v0, v1, v2 = (tris[:, k].astype(np.float64) for k in range(3))
    e1, e2 = v1 - v0, v2 - v0
    p = np.cross(d[None], e2)
    det = np.einsum("ij,ij->i", e1, p)
    with np.errstate(divide="ignore", invalid="ignore"):
        inv = 1.0 / det
        tv = o[None] - v0
        u = np.einsum("ij,ij->i", tv, p) * inv
        q = np.cross(tv, e1)
        v = (q @ d) * inv
        t = np.einsum("ij,ij->i", e2, q) * inv
    # accepted within 2e-5 of an edge: a near-tie classifier, looser than either float test
    ok = (u >= -2e-5) & (v >= -2e-5) & (u + v <= 1 + 2e-5) & (t >= 0) & np.isfinite(t)
    return np.where(ok, t, np.inf)


def test_microbench_rays_match_reference(ref, tmp_path):
    n_tris = 1 << 20
    cp, sp = scenes.tri_soup(str(tmp_path / "soup"), n_tris=n_tris)
    tris = scenes.tri_soup_arrays(n_tris)
    o_all, d_all = scenes.microbench_rays(1 << 24)  # the microbench's 16M rays
    rng = np.random.default_rng(11)
    half = 1 << 23
    sel = np.concatenate([np.sort(rng.choice(half, 32768, replace=False)),
                          half + np.sort(rng.choice(half, 32768, replace=False))])
    o, d = np.ascontiguousarray(o_all[sel]), np.ascontiguousarray(d_all[sel])
    del o_all, d_all
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    gobj, gt = ctx.trace_rays(o, d)
    R = ref.ref_open(cp, sp)
    robj, rt = R.intersect(o, d, threads=THREADS)
    assert (robj >= 0).mean() > 0.3  # both halves hit the soup often
    # closest hit: the same object except where two hits are within float rounding of each other
    diff = np.nonzero(gobj != robj)[0]
    assert diff.size <= 1e-3 * len(o), f"{diff.size} of {len(o)} rays hit another object"
    for i in diff:
        bf = _fp64_hits(o[i], d[i], tris)
        t_best = bf.min()
        assert np.isfinite(t_best)
        for obj_, t_ in ((gobj[i], gt[i]), (robj[i], rt[i])):
            assert obj_ >= 0 and abs(bf[obj_] - t_best) <= 1e-5 * t_best, (i, obj_, bf[obj_], t_best)
    # t of every GPU hit within 1e-5 of the FP64 solve of the same triangle, except where the
    # reference's own float t (glm's cofactor inverse, Triangle.cpp:38-40) is off by as much: at
    # short distances the inverse's cancellation costs relative accuracy, and there the GPU's t
    # is the reference's to the bit
    hit = np.nonzero(gobj >= 0)[0]
    v0, v1, v2 = (tris[gobj[hit], k].astype(np.float64) for k in range(3))
    e1, e2 = v1 - v0, v2 - v0
    dd = d[hit].astype(np.float64)
    pp = np.cross(dd, e2)
    det = np.einsum("ij,ij->i", e1, pp)
    q = np.cross(o[hit].astype(np.float64) - v0, e1)
    t64 = np.einsum("ij,ij->i", e2, q) / det
    rel = np.abs(gt[hit] - t64) / np.abs(t64)
    same_ref = (gobj[hit] == robj[hit]) & (gt[hit].view(np.uint32) == rt[hit].view(np.uint32))
    print(f"closest hit: {diff.size} id differences (near-ties), t within 1e-5 of FP64 on {(rel <= 1e-5).mean():.5%} "
          f"of {hit.size} hits, max {rel.max():.2e}; t bit-equal to the reference on {same_ref.mean():.4%}")
    assert np.all((rel <= 1e-5) | same_ref)
    assert (rel <= 1e-5).mean() >= 0.999
    # any hit at the microbench's random tmax: U(0, 2 t_closest) on hits, U(0, 4) on misses
    u = rng.random(len(o)).astype(np.float32)
    tmax = np.where(gobj >= 0, 2.0 * gt * u, 4.0 * u).astype(np.float32)
    tmin = np.zeros(len(o), np.float32)
    ign = np.full(len(o), -1, np.int32)
    gocc = ctx.trace_rays(o, d, any_hit=True, tmin=tmin, tmax=tmax, ignore=ign)
    rocc = R.intersect_test_mt(o, d, tmin, tmax, ign, threads=THREADS)
    assert 0.1 < rocc.mean() < 0.9
    assert np.array_equal(gocc, rocc), f"{(gocc != rocc).sum()} any-hit answers differ"


# ---- Cornell box at its full configuration ----------------------------------------------------------

def test_cornell_full_config_relmse_matches_reference(ref, tmp_path):
    """relMSE of 64-spp images against a 16384-spp plain GPU render: the GPU's within 2% of the
    reference CPU's.  Each side's relMSE is the mean over sixteen independent 64-spp images (sample
    runs 0-63, 64-127, ...): one 64-spp image's relMSE varies by about 2.3% (standard deviation)
    from one sample run to the next on this scene, so single draws could not resolve a 2% bar,
    while the difference of two 16-run means has a standard deviation near 0.8%.  Per-pixel means
    of all 1024 samples within 3 standard errors."""
    spp, runs = 64, 16
    cp, sp = scenes.cornell(str(tmp_path / "c"), spp=spp * runs)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    # converged image from a disjoint sample range
    conv, _ = _gpu_film(ctx, 1 << 22, 16384)
    Rimg = conv / 16384
    g_runs, g_s, g_q = [], 0.0, 0.0
    for k in range(runs):
        s, q = _gpu_film(ctx, spp * k, spp)
        g_runs.append(_relmse(s / spp, Rimg))
        g_s, g_q = g_s + s, g_q + q
    R = ref.ref_open(cp, sp)
    S, Q, secs = R.render_region_groups(0, 0, R.W, R.H, spp, threads=THREADS)
    c_runs = [_relmse(S[k] / spp, Rimg) for k in range(runs)]
    g_rel, c_rel = float(np.mean(g_runs)), float(np.mean(c_runs))
    print(f"relMSE vs 16384 spp: GPU {g_rel:.6f} {np.round(g_runs, 6)}, reference {c_rel:.6f} {np.round(c_runs, 6)} "
          f"(reference {secs:.1f} s on {THREADS} threads)")
    assert abs(g_rel / c_rel - 1) <= 0.02
    z, gm, cm, var = _zscores(g_s, g_q, spp * runs, S.sum(0), Q, spp * runs)
    assert (np.abs(z) > 3).mean() <= 0.01
    assert abs(gm.mean() - cm.mean()) <= 3 * np.sqrt(var.sum()) / var.size


# ---- many-material scene at 1080p ----------------------------------------------------------------

def test_many_material_band_matches_reference(ref, tmp_path):
    spp = 16
    cp, sp = scenes.many_material(str(tmp_path / "mm"), spp=spp)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    s, q = _gpu_film(ctx, 0, spp)
    y0, y1 = 508, 572
    R = ref.ref_open(cp, sp)
    rs, rq, secs = R.render_region(0, y0, R.W, y1, threads=THREADS)
    z, gm, cm, var = _zscores(s[y0:y1], q[y0:y1], spp, rs, rq, spp)
    frac = float((np.abs(z) > 3).mean())
    print(f"band rows {y0}..{y1 - 1}: |z| > 3 on {frac:.4%} of pixel channels; means {gm.mean():.5f} vs {cm.mean():.5f} "
          f"(reference {secs:.1f} s)")
    assert frac <= 0.01
    assert abs(gm.mean() - cm.mean()) <= 3 * np.sqrt(var.sum()) / var.size


# ---- slit-lit room ---------------------------------------------------------------------------------

@pytest.mark.parametrize("accel,hf,w,h,spp", [("BVH", 512, 96, 54, 256), ("Brute", 16, 48, 27, 256)])
def test_slit_room_plain_matches_reference(ref, accel, hf, w, h, spp, tmp_path):
    cp, sp = scenes.slit_room(str(tmp_path / f"slit_{accel}"), width=w, height=h, spp=spp, depth=12, hf_res=hf,
                              accel=accel)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    s, q = _gpu_film(ctx, 0, spp)
    R = ref.ref_open(cp, sp)
    rs, rq, secs = R.render_region(0, 0, w, h, threads=THREADS)
    z, gm, cm, var = _zscores(s, q, spp, rs, rq, spp)
    frac = float((np.abs(z) > 3).mean())
    print(f"slit room {accel} hf {hf}: |z| > 3 on {frac:.4%}; means {gm.mean():.5f} vs {cm.mean():.5f} (reference {secs:.1f} s)")
    assert frac <= 0.01
    assert abs(gm.mean() - cm.mean()) <= 3 * np.sqrt(var.sum()) / var.size


def test_guided_estimator_is_unbiased_on_slit_room(tmp_path):
    """The guided tracer's image agrees with the plain tracer's on the slit room (the scene the
    equal-time comparison uses): image means within 3 standard errors and 1e-3 relative at 16384
    guided and 65536 plain spp, and per-pixel z-scores no worse than a plain-vs-plain control."""
    w, h = 32, 24
    cp, sp = scenes.slit_room(str(tmp_path / "slit"), width=w, height=h, spp=64, depth=12, hf_res=512)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    tiles = ((w + 7) // 8) * ((h + 7) // 8) * 64

    def film(integ, s0, n, wave_spp):
        p = ctx.render_params()
        p.integrator, p.sample_begin, p.sample_count, p.wave_paths = integ, s0, n, tiles * wave_spp
        ctx.film_clear()
        ctx.render(p)
        s, _ = ctx.film()
        return s.astype(np.float64), ctx.film_m2().astype(np.float64)

    n_plain, n_guided = 16 * 4096, 4 * 4096
    ps, pq = film(N.INTEGRATOR_PATH, 0, n_plain, 1024)
    cs, cq = film(N.INTEGRATOR_PATH, 1 << 20, n_guided, 1024)
    ctx.guide_config(2e-3, 0.7, 2, 4)
    ctx.guide_levels(0)
    gs, gq = film(N.INTEGRATOR_GUIDED, 0, n_guided, 64)
    assert ctx.guide_stats()[2] > 0
    zc, _, _, _ = _zscores(cs, cq, n_guided, ps, pq, n_plain)
    zg, gm, pm, var = _zscores(gs, gq, n_guided, ps, pq, n_plain)
    se = np.sqrt(var.sum()) / var.size
    print(f"slit room means: guided {gm.mean():.6f}, plain {pm.mean():.6f} (se {se:.2e}); "
          f"|z|<3: guided {np.mean(np.abs(zg) < 3):.4f}, control {np.mean(np.abs(zc) < 3):.4f}")
    assert abs(gm.mean() - pm.mean()) <= max(3 * se, 1e-3 * pm.mean())
    assert np.mean(np.abs(zg) < 3) >= np.mean(np.abs(zc) < 3) - 0.02
    assert abs(np.mean(zg)) < 0.2
