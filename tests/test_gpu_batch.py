"""Batched multi-job rendering (c2g_batch_*): replayed wave graphs on concurrent streams render the
same films as one-job-at-a-time c2g_render calls with the same wave size."""
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


def test_batch_matches_individual_renders(tmp_path):
    jobs = [_job(tmp_path, "c1", scenes.cornell, N.INTEGRATOR_PATH, 16, width=32, height=32),
            _job(tmp_path, "c2", scenes.cornell, N.INTEGRATOR_PATH, 12, width=40, height=24),
            _job(tmp_path, "mb", scenes.material_box, N.INTEGRATOR_PATH, 8, width=48, height=48)]
    wave_paths = 4096
    solo = [_solo(c, p, wave_paths) for c, p in jobs]
    b = Batch(0)
    for c, p in jobs:
        c.film_clear()
        b.add(c, p)
    b.tune(wave_paths, 2)
    st = b.run()
    assert st.jobs == 3
    assert st.paths == sum(p.width * p.height * p.sample_count for _, p in jobs)
    assert st.graph_launches > 3 and st.streams == 2
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
        b.tune(1 << 20, 0)   # at least one stream
    q = N.RenderParams.from_buffer_copy(p)
    q.sample_count = 0
    c2, _ = _job(tmp_path, "c2", scenes.cornell, N.INTEGRATOR_PATH, 4, width=16, height=16)
    with pytest.raises(N.C2GError):
        b.add(c2, q)         # a job renders at least one sample
    b.close()
