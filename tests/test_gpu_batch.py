"""Batched multi-job rendering (c2g_batch_*): the whole batch as one graph launch with device-side
wave loops, and replayed per-job wave graphs on concurrent streams, render the same films as
one-job-at-a-time c2g_render calls with the same wave size."""
import numpy as np
import pytest

from crystal2_gb300 import Batch, Context, scenes
from crystal2_gb300 import _native as N

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module", autouse=True)
def _built():
    from crystal2_gb300 import build
    build.build()


def _job(tmp_path, name, make, integrator, spp, **kw):
    cp, sp = make(str(tmp_path / name), **kw)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    p = ctx.render_params()
    p.integrator = integrator
    p.sample_begin = 0
    p.sample_count = spp
    return ctx, p


def _solo(ctx, p, wave_paths):
    q = N.RenderParams.from_buffer_copy(p)
    nslots = ((q.width + 7) // 8) * ((q.height + 7) // 8) * 64
    spw = max(1, min(q.sample_count, wave_paths // nslots))
    while q.sample_count % spw:
        spw -= 1
    q.wave_paths = spw * nslots
    ctx.film_clear()
    ctx.render(q)
    return ctx.film()


@pytest.mark.parametrize("streams,lanes", [(2, None), (0, 8), (0, 1), (0, 0)])
def test_batch_matches_individual_renders(tmp_path, streams, lanes):
    jobs = [_job(tmp_path, "c1", scenes.cornell, N.INTEGRATOR_PATH, 16, width=32, height=32),
            _job(tmp_path, "c2", scenes.cornell, N.INTEGRATOR_PATH, 12, width=40, height=24),
            _job(tmp_path, "mb", scenes.material_box, N.INTEGRATOR_PATH, 8, width=48, height=48)]
    wave_paths = 4096
    solo = [_solo(c, p, wave_paths) for c, p in jobs]
    b = Batch(0)
    for c, p in jobs:
        c.film_clear()
        b.add(c, p)
    b.tune(wave_paths, streams)
    if lanes is not None:
        b.set_lanes(lanes)  # one chain per job (0), all jobs in one chain (1), or the default 8
    st = b.run()
    assert st.jobs == 3
    assert st.paths == sum(p.width * p.height * p.sample_count for _, p in jobs)
    assert st.streams == streams
    # one launch for the whole batch, or one per wave
    assert st.graph_launches == 1 if streams == 0 else st.graph_launches > 3
    for (c, p), (s_ref, w_ref) in zip(jobs, solo):
        s, w = c.film()
        assert np.array_equal(w, w_ref)
        assert np.array_equal(s, s_ref)
    lat = [b.latency_ms(i) for i in range(3)]
    assert all(0 < x <= st.seconds * 1e3 + 1e-3 for x in lat)
    assert st.latency_max_ms == pytest.approx(max(lat))
    # a second run adds the same samples again
    st2 = b.run()
    s, w = jobs[0][0].film()
    assert np.array_equal(w, 2 * solo[0][1])
    b.close()


def test_batch_guided_job_and_autotune(tmp_path):
    jobs = [_job(tmp_path, "g", scenes.cornell, N.INTEGRATOR_GUIDED, 32, width=32, height=32),
            _job(tmp_path, "p", scenes.cornell, N.INTEGRATOR_PATH, 32, width=32, height=32)]
    b = Batch(0)
    for c, p in jobs:
        c.film_clear()
        b.add(c, p)
    best = b.autotune(wave_paths=(2048, 8192), streams=(1, 2), trial_spp=4)
    assert best > 0
    st = b.run()
    assert st.wave_paths in (2048, 8192) and st.streams in (1, 2)
    assert jobs[0][0].guide_stats()[2] > 0  # the guided job trained inside its graphs
    g = jobs[0][0].image().astype(np.float64)
    p = jobs[1][0].image().astype(np.float64)
    # same scene, same sample count: the guided estimate agrees with the plain one in the mean
    assert abs(g.mean() - p.mean()) < 0.05 * p.mean()
    b.close()


def test_batch_rejects_bad_input(tmp_path):
    c, p = _job(tmp_path, "c", scenes.cornell, N.INTEGRATOR_PATH, 4, width=16, height=16)
    b = Batch(0)
    b.add(c, p)
    with pytest.raises(N.C2GError):
        b.add(c, p)          # a context joins a batch once
    with pytest.raises(N.C2GError):
        b.tune(1 << 20, -1)  # 0 (one graph launch) or 1..32 streams
    with pytest.raises(N.C2GError):
        b.set_trace(3, 128)  # node width 2 or 4
    with pytest.raises(N.C2GError):
        b.set_trace(4, 96)   # block of 64, 128 or 256 threads
    q = N.RenderParams.from_buffer_copy(p)
    q.sample_count = 0
    c2, _ = _job(tmp_path, "c2", scenes.cornell, N.INTEGRATOR_PATH, 4, width=16, height=16)
    with pytest.raises(N.C2GError):
        b.add(c2, q)         # a job renders at least one sample
    b.close()


@pytest.mark.parametrize("streams", [0, 2])
def test_batch_rejects_direct_lighting(tmp_path, streams):
    """The direct lighting integrator walks pass-through hops with a host-side queue check, so it
    cannot run inside batch graphs: both modes refuse it with an error, not a wrong film."""
    c, p = _job(tmp_path, "d", scenes.cornell, N.INTEGRATOR_DIRECT, 4, width=16, height=16)
    b = Batch(0)
    b.add(c, p)
    b.tune(4096, streams)
    with pytest.raises(N.C2GError):
        b.run()
    b.close()


def test_batch_search_one_launch_guided(tmp_path):
    """The coordinate search picks a configuration from every dimension's candidates; the chosen one
    renders a guided and a plain job in one graph launch, the guided job training inside it."""
    jobs = [_job(tmp_path, "g", scenes.cornell, N.INTEGRATOR_GUIDED, 32, width=32, height=32),
            _job(tmp_path, "p", scenes.cornell, N.INTEGRATOR_PATH, 32, width=32, height=32),
            _job(tmp_path, "m", scenes.material_box, N.INTEGRATOR_PATH, 16, width=24, height=24)]
    b = Batch(0)
    for c, p in jobs:
        c.film_clear()
        b.add(c, p)
    best = b.search(wave_paths=(2048, 8192), streams=(0, 2), traversal=(4, 2), trace_block=(128, 64, 256), trial_spp=4)
    assert best > 0
    b.tune(8192, 0)  # whatever the search chose, run the one-launch mode with its traversal choice
    st = b.run()
    assert st.graph_launches == 1 and st.traversal in (2, 4) and st.trace_block in (64, 128, 256)
    assert jobs[0][0].guide_stats()[2] > 0
    for c, p in jobs:
        s, w = c.film()
        assert np.all(w == p.sample_count)
    g = jobs[0][0].image().astype(np.float64)
    pl = jobs[1][0].image().astype(np.float64)
    assert abs(g.mean() - pl.mean()) < 0.05 * pl.mean()
    assert st.latency_p50_ms <= st.latency_p90_ms <= st.latency_max_ms
    b.close()


@pytest.mark.parametrize("traversal,block", [(2, 64), (4, 256)])
def test_batch_trace_settings_keep_films(tmp_path, traversal, block):
    """Traversal variant and block size change how rays are traced, not what they hit: the films equal
    the default configuration's."""
    ref = None
    for tv, bl in ((4, 128), (traversal, block)):
        c, p = _job(tmp_path, f"c{tv}{bl}", scenes.material_box, N.INTEGRATOR_PATH, 8, width=32, height=32)
        b = Batch(0)
        c.film_clear()
        b.add(c, p)
        b.tune(4096, 0)
        b.set_trace(tv, bl)
        b.run()
        s, w = c.film()
        b.close()
        if ref is None:
            ref = (s, w)
        else:
            assert np.array_equal(w, ref[1])
            # the binary and four-wide trees give the same closest hits up to near-ties
            close = np.isclose(s, ref[0], rtol=1e-4, atol=1e-6)
            assert close.mean() > 0.98


def test_batch_search_skips_wave_sizes_that_do_not_fit(tmp_path):
    """With a memory cap per context, a wave size whose buffers do not fit fails its trial with
    C2G_ERR_OOM: the search releases the buffers, keeps the candidate that fits and the batch runs."""
    jobs = []
    for i in range(2):
        cp, sp = scenes.cornell(str(tmp_path / f"c{i}"), width=32, height=32, spp=256)
        ctx = Context(0, mem_limit_bytes=64 << 20)
        ctx.load(cp, sp, tree=N.TREE_SAH)
        p = ctx.render_params()
        p.sample_begin, p.sample_count = 0, 256
        jobs.append((ctx, p))
    b = Batch(0)
    for c, p in jobs:
        c.film_clear()
        b.add(c, p)
    # 4096 paths per wave fit (about 2 MB of wave buffers per job); 2^20 do not (256 samples of 1024
    # pixel slots: about 100 MB)
    best = b.search(wave_paths=(4096, 1 << 20), streams=(0,), traversal=(4,), trace_block=(128,), trial_spp=256)
    assert best > 0
    st = b.run()
    assert st.wave_paths == 4096
    for c, p in jobs:
        s, w = c.film()
        assert np.all(w == p.sample_count) and np.isfinite(s).all()
    b.close()
