"""CPU checks of the guiding-network oracle (oracle/guide_oracle.py) and of the guide C ABI's host
behaviour.  The oracle's analytic gradient is pinned against central finite differences, the BF16
rounding helper against known bit patterns, and the mixture density against numerical integration
over the sphere."""
import numpy as np
import pytest

from crystal2_gb300 import _native as N
from oracle import guide_oracle as G


def test_param_layout_matches_c_abi():
    assert G.N_PARAMS == N.GUIDE_PARAMS == 16624
    assert G.N_OUT == N.GUIDE_OUTPUTS


def test_bf16_rounding_known_values():
    v = np.array([1.0, 1.00390625, 1.005859375, 3.14159265, -2.5e-3, 0.0], np.float32)
    r = G.bf16(v)
    # 1 + 2^-8 is a tie between 1 and 1 + 2^-7: ties to even -> 1.0; 1.005859375 rounds up
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == 1.0078125
    assert r[3] == 3.140625
    assert abs(r[4] - -2.5e-3) <= 2.5e-3 * 2 ** -8
    assert r[5] == 0.0


def test_analytic_gradient_matches_finite_differences():
    assert G.finite_difference_check(seed=0) < 1e-4
    assert G.finite_difference_check(seed=5, m=8) < 1e-4


def test_mixture_pdf_integrates_to_one():
    params = G.init_params(3, out_scale=3.0)
    x, n, wo, _, _, _ = G.random_samples(4, seed=9)
    out, _ = G.forward(params, G.encode(x, n, wo, (-1, -1, -1), (1, 1, 1)), bf16_mode=False)
    # midpoint quadrature in (cos theta, phi): the measure is uniform in those coordinates
    nt, npf = 1200, 600
    ct = -1 + (np.arange(nt) + 0.5) * 2 / nt
    ph = (np.arange(npf) + 0.5) * 2 * np.pi / npf
    C, P = np.meshgrid(ct, ph, indexing="ij")
    S = np.sqrt(1 - C ** 2)
    dirs = np.stack([S * np.cos(P), S * np.sin(P), C], -1).reshape(-1, 3)
    for j in range(out.shape[0]):
        o = np.repeat(out[j:j + 1], dirs.shape[0], axis=0)
        p = G.mixture_pdf(o, dirs)
        integral = p.sum() * (2 / nt) * (2 * np.pi / npf)
        assert abs(integral - 1) < 2e-3, integral


def test_guide_calls_refused_on_host_only_context():
    from crystal2_gb300 import Context
    ctx = Context(device=-1)
    with pytest.raises(N.C2GError) as e:
        ctx.guide_params()
    assert e.value.code == N.C2G_ERR_STATE
    with pytest.raises(N.C2GError) as e:
        ctx.guide_reset((0, 0, 0), (1, 1, 1))
    assert e.value.code == N.C2G_ERR_STATE
    with pytest.raises(N.C2GError) as e:
        ctx.guide_config(learning_rate=-1.0)
    assert e.value.code == N.C2G_ERR_INVALID
