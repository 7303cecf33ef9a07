"""GPU checks of the learned guiding proposal through the C ABI.

* the tensor-core forward pass and the fused backward kernel against the FP64 oracle
  (oracle/guide_oracle.py, BF16 rounding emulated at the kernels' storage points);
* online training lowers the weighted negative log-likelihood on the slit-lit room;
* the guided estimator is unbiased: its image mean agrees with the plain path tracer's;
* the trained proposal lowers the error at equal sample count on the slit-lit room (512 spp).
"""
import numpy as np
import pytest

from crystal2_gb300 import Context, scenes
from crystal2_gb300 import _native as N
from oracle import guide_oracle as G

pytestmark = pytest.mark.gpu

BOX_LO, BOX_HI = (-1.0, -1.0, -1.0), (1.0, 1.0, 1.0)


@pytest.fixture(scope="module", autouse=True)
def _built():
    from crystal2_gb300 import build
    build.build()


def _guide_ctx(seed=0, out_scale=1.0):
    ctx = Context(0)
    ctx.guide_reset(BOX_LO, BOX_HI, seed=7)
    params = G.init_params(seed, out_scale=out_scale).astype(np.float32)
    ctx.guide_set_params(params)
    return ctx, params


def test_params_round_trip():
    ctx, params = _guide_ctx()
    assert np.array_equal(ctx.guide_params(), params)


def test_forward_matches_oracle():
    ctx, params = _guide_ctx(seed=1)
    x, n, wo, _, _, _ = G.random_samples(1000, seed=2)
    out = ctx.guide_eval(np.concatenate([x, n, wo], 1))
    ref, _ = G.forward(params.astype(np.float64), G.encode(x, n, wo, BOX_LO, BOX_HI), bf16_mode=True)
    ref = ref[:, :G.N_OUT]
    scale = np.abs(ref).max()
    # BF16 activations: an activation that rounds the other way moves an output by ~2^-8 of its size
    assert np.abs(out - ref).max() < 2e-2 * scale
    assert np.sqrt(np.mean((out - ref) ** 2)) < 2e-3 * scale
    # and the mixture densities it implies agree closely
    wi = G.random_samples(1000, seed=3)[3].astype(np.float64)
    q_gpu = G.mixture_pdf(out.astype(np.float64), wi)
    q_ref = G.mixture_pdf(ref, wi)
    assert np.median(np.abs(q_gpu / q_ref - 1)) < 1e-2


@pytest.mark.parametrize("n", [1, 127, 128, 129, 257, 2000])
def test_forward_tiles_match_oracle(n):
    """The tensor-core forward pass runs 128-row tiles, two per CTA: partial last tiles, a single
    row and counts around the tile size give the oracle's outputs row for row."""
    ctx, params = _guide_ctx(seed=6)
    x, nn, wo, _, _, _ = G.random_samples(n, seed=7)
    out = ctx.guide_eval(np.concatenate([x, nn, wo], 1))
    ref, _ = G.forward(params.astype(np.float64), G.encode(x, nn, wo, BOX_LO, BOX_HI), bf16_mode=True)
    ref = ref[:, :G.N_OUT]
    assert out.shape == ref.shape
    scale = np.abs(ref).max()
    assert np.abs(out - ref).max() < 2e-2 * scale
    # rows are independent: the first rows of a longer batch are the same numbers
    if n > 1:
        head = ctx.guide_eval(np.concatenate([x[:1], nn[:1], wo[:1]], 1))
        assert np.array_equal(head[0], out[0])


@pytest.mark.parametrize("m", [37, 4096])
def test_gradient_matches_oracle(m):
    ctx, params = _guide_ctx(seed=4)
    x, n, wo, wi, w, pb = G.random_samples(m, seed=5)
    samples = np.concatenate([x, n, wo, wi, w[:, None], pb[:, None]], 1)
    g, loss = ctx.guide_gradient(samples)
    enc = G.encode(x, n, wo, BOX_LO, BOX_HI)
    gr, lsum, wsum = G.nll_gradient(params.astype(np.float64), enc, wi, w, pb, bf16_mode=True)
    assert abs(loss - lsum / wsum) < 2e-3 * max(1.0, abs(lsum / wsum))
    o = 0
    for l, (k, nn) in enumerate(G.SHAPES):
        for part, size in (("W", k * nn), ("b", nn)):
            a, b = g[o:o + size].astype(np.float64), gr[o:o + size]
            o += size
            rel = np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-12)
            cos = a @ b / max(np.linalg.norm(a) * np.linalg.norm(b), 1e-30)
            assert rel < 3e-2 and cos > 0.999, (l, part, rel, cos)
    # the padded output columns get no gradient
    pad = np.array([G._is_pad(i) for i in range(G.N_PARAMS)])
    assert np.all(g[pad] == 0)


def _slit(tmp_path, w=64, h=48, spp=64, integ="PathTracer", hf=64):
    cp, sp = scenes.slit_room(str(tmp_path / "slit"), width=w, height=h, spp=spp, depth=12, hf_res=hf, integrator=integ)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    return ctx


def _render(ctx, integrator, spp, wave_spp, sample_begin=0, seed=0):
    p = ctx.render_params()
    p.integrator = integrator
    p.sample_begin = sample_begin
    p.sample_count = spp
    p.seed = seed
    tiles = ((p.width + 7) // 8) * ((p.height + 7) // 8) * 64
    p.wave_paths = tiles * wave_spp
    ctx.film_clear()
    ctx.render(p)
    return ctx.image().astype(np.float64)


def test_training_lowers_loss(tmp_path):
    """One Adam step per wave, so each reported loss is that of the wave's whole batch (with
    several steps per wave each step sees one window of the batch and its loss is noisier)."""
    ctx = _slit(tmp_path)
    ctx.guide_config(learning_rate=5e-3, bsdf_fraction=0.5, warmup_waves=1000, train_steps=1)
    losses = []
    for k in range(48):
        _render(ctx, N.INTEGRATOR_GUIDED, 2, 2, sample_begin=2 * k)
        loss, records, steps = ctx.guide_stats()
        assert records > 0
        losses.append(loss)
    assert steps == 48
    first, last = np.mean(losses[:3]), np.mean(losses[-6:])
    assert np.all(np.isfinite(losses))
    assert last < first - 0.05, losses


def _z(a, m2a, b, m2b, n):
    va = np.maximum(m2a[..., :3] / n - a ** 2, 0) / n
    vb = np.maximum(m2b[..., :3] / n - b ** 2, 0) / n
    se = np.sqrt(va + vb)
    d = a - b
    return d[se > 0] / se[se > 0], d, se


def test_guided_estimator_is_unbiased(tmp_path):
    """Guided vs plain per-pixel z-scores behave like plain vs plain (an independent sample range):
    heavy-tailed caustic paths make both deviate from N(0, 1) in the same way."""
    cp, sp = scenes.cornell(str(tmp_path / "c"), width=32, height=32, spp=1024)
    ctx = Context(0)
    ctx.load(cp, sp, tree=N.TREE_SAH)
    ctx.guide_config(learning_rate=5e-3, bsdf_fraction=0.3, warmup_waves=2, train_steps=2)
    n = 1024
    plain = _render(ctx, N.INTEGRATOR_PATH, n, 16)
    m2p = ctx.film_m2()
    control = _render(ctx, N.INTEGRATOR_PATH, n, 16, sample_begin=5000)
    m2c = ctx.film_m2()
    guided = _render(ctx, N.INTEGRATOR_GUIDED, n, 16)
    m2g = ctx.film_m2()
    assert ctx.guide_stats()[2] > 0
    zc, _, _ = _z(control, m2c, plain, m2p, n)
    zg, d, se = _z(guided, m2g, plain, m2p, n)
    assert abs(d.mean()) < 3 * np.sqrt((se ** 2).sum()) / d.size
    assert np.mean(np.abs(zg) < 3) > np.mean(np.abs(zc) < 3) - 0.02
    assert abs(np.mean(zg)) < 0.15


def test_guided_lowers_error_on_slit_room(tmp_path):
    ctx = _slit(tmp_path)
    ref = _render(ctx, N.INTEGRATOR_PATH, 4096, 256, sample_begin=100000)

    def relmse(img):
        return float(np.mean((img - ref) ** 2 / (ref ** 2 + 1e-2)))

    plain = relmse(_render(ctx, N.INTEGRATOR_PATH, 512, 4))
    ctx.guide_config(learning_rate=5e-3, bsdf_fraction=0.5, warmup_waves=4, train_steps=4)
    guided = relmse(_render(ctx, N.INTEGRATOR_GUIDED, 512, 4))
    print(f"relMSE plain {plain:.4f} guided {guided:.4f}")
    assert guided < plain
