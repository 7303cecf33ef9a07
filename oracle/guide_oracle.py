"""FP64 CPU oracle of the guiding network: encoding, forward pass, mixture density and the gradient
of the weighted negative log-likelihood the training kernel minimises.

TEST INFRASTRUCTURE ONLY: imported by tests/ to check the CUDA forward/backward kernels.  Product
code never imports this module.

The reference has no learned guiding, so there is no reference function to follow; this module
restates the network defined by the library's C ABI (include/c2g.h, "learned guiding proposal"):

* input: p = clamp((x - lo) * inv, 0, 1) per axis (FP32), then sin/cos(pi 2^f p) for f = 0..11
  (axis-major, sin before cos; octaves above the first by the FP32 double-angle recurrence the
  kernels use), then the normal, the outgoing direction and two zeros (80 values);
* layers 80->64->64->64->48 with ReLU after the hidden layers; parameters are one flat vector,
  per layer W (K x N row-major) then b (N);
* outputs 5 per lobe (8 lobes): mean direction (normalised), concentration softplus(k) + 0.05
  (capped at 500), weight softmax(logit); density q = sum_k w_k vMF(wi; mu_k, kappa_k); output 40
  is the selection logit s: the sampler draws from q with probability c = 0.05 + 0.75 sigmoid(s)
  and from the BSDF otherwise, so the training loss is -w log q_mix, q_mix = (1 - c) p_bsdf + c q.

``bf16=True`` rounds at the points where the kernels store BF16 (encoded inputs, weights, hidden
activations, the output gradient and the back-propagated deltas); ``bf16=False`` is plain FP64,
which ``finite_difference_check`` uses to pin the analytic gradient.
"""
from __future__ import annotations

import numpy as np

N_IN, HIDDEN, N_OUT, N_OUT_PAD, LOBES, FREQS = 80, 64, 41, 48, 8, 12
SHAPES = [(N_IN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, HIDDEN), (HIDDEN, N_OUT_PAD)]
KAPPA_MAX = 500.0            # vMF concentration cap
SEL_MIN, SEL_SPAN = 0.05, 0.75  # selection probability c in [0.05, 0.8]
N_PARAMS = sum(k * n + n for k, n in SHAPES)


def bf16(a) -> np.ndarray:
    """Round to the nearest BF16 (ties to even), returned as float64."""
    f = np.ascontiguousarray(a, np.float32)
    u = f.view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32).astype(np.float64)


def unpack(params: np.ndarray):
    """Flat vector -> [(W K x N, b N)] in float64."""
    out, o = [], 0
    p = np.asarray(params, np.float64)
    for k, n in SHAPES:
        W = p[o:o + k * n].reshape(k, n)
        o += k * n
        b = p[o:o + n]
        o += n
        out.append((W, b))
    return out


def pack(layers) -> np.ndarray:
    return np.concatenate([np.concatenate([W.ravel(), b]) for W, b in layers]).astype(np.float64)


def encode(x, n, wo, lo, hi) -> np.ndarray:
    """(m, 80) network inputs.  Positions are normalised in FP32 as the kernels do."""
    x = np.asarray(x, np.float32)
    lo = np.asarray(lo, np.float32)
    ext = np.asarray(hi, np.float32) - lo
    inv = np.where(ext > 0, np.float32(1) / np.where(ext > 0, ext, 1), np.float32(1)).astype(np.float32)
    p = np.clip((x - lo) * inv, 0, 1).astype(np.float64)
    m = x.shape[0]
    enc = np.zeros((m, N_IN))
    for a in range(3):
        # sin/cos(pi p) rounded to FP32, then the FP32 double-angle recurrence of the kernels:
        # sin 2u = 2 sin u cos u, cos 2u = (cos u - sin u)(cos u + sin u)
        s = np.sin(np.pi * p[:, a]).astype(np.float32)
        c = np.cos(np.pi * p[:, a]).astype(np.float32)
        for f in range(FREQS):
            enc[:, a * 2 * FREQS + 2 * f] = s
            enc[:, a * 2 * FREQS + 2 * f + 1] = c
            s, c = (np.float32(2) * s * c).astype(np.float32), ((c - s) * (c + s)).astype(np.float32)
    enc[:, 72:75] = np.asarray(n, np.float64)
    enc[:, 75:78] = np.asarray(wo, np.float64)
    return enc


def forward(params, enc, bf16_mode=True):
    """Returns (outputs (m, 48), activations [a0, h1, h2, h3]) of the MLP."""
    layers = unpack(params)
    r = bf16 if bf16_mode else (lambda v: np.asarray(v, np.float64))
    acts = [r(enc)]
    h = acts[0]
    for l, (W, b) in enumerate(layers):
        z = h @ r(W) + b
        if l < 3:
            h = r(np.maximum(z, 0.0))
            acts.append(h)
        else:
            out = z
    return out, acts


def softplus(x):
    return np.where(x > 15, x, np.log1p(np.exp(np.minimum(x, 15))))


def lobes(out):
    """(mu (m, 8, 3), kappa (m, 8), w (m, 8)) from raw outputs."""
    o = out[:, :LOBES * 5].reshape(-1, LOBES, 5)
    m = o[:, :, :3]
    ln = np.linalg.norm(m, axis=2, keepdims=True)
    mu = np.where(ln > 1e-12, m / np.maximum(ln, 1e-300), np.array([0.0, 1.0, 0.0]))
    kappa = np.minimum(softplus(o[:, :, 3]) + 0.05, KAPPA_MAX)
    lg = o[:, :, 4]
    e = np.exp(lg - lg.max(axis=1, keepdims=True))
    w = e / e.sum(axis=1, keepdims=True)
    return mu, kappa, w


def vmf_pdf(mu, kappa, wi):
    c = np.einsum("mkj,mj->mk", mu, wi)
    return kappa / (2 * np.pi * (-np.expm1(-2 * kappa))) * np.exp(kappa * (c - 1))


def mixture_pdf(out, wi):
    mu, kappa, w = lobes(out)
    return (w * vmf_pdf(mu, kappa, np.asarray(wi, np.float64))).sum(axis=1)


def select_prob(s):
    return SEL_MIN + SEL_SPAN / (1 + np.exp(-s))


def nll_gradient(params, enc, wi, weight, pb, bf16_mode=True, clamp=1e3):
    """(grad (N_PARAMS,), loss_sum, weight_sum) of sum_j w_j * -log q_mix(wi_j).

    Output-gradient formulas, with rho = c q / q_mix: d log q_mix / d logit_k = rho (r_k - w_k)
    (r = posterior lobe share); d log q_mix / d kraw_k = rho r_k (1/kappa - 2 e^-2kappa /
    (1 - e^-2kappa) + mu.wi - 1) sigmoid(kraw) (zero where kappa is capped); d log q_mix / d m_k =
    rho r_k kappa (wi - mu (mu.wi)) / |m_k|; d log q_mix / d s = (q - p_bsdf) 0.75 sigmoid'(s) / q_mix.
    """
    r = bf16 if bf16_mode else (lambda v: np.asarray(v, np.float64))
    layers = unpack(params)
    out, acts = forward(params, enc, bf16_mode)
    wi = np.asarray(wi, np.float64)
    wgt = np.asarray(weight, np.float64)
    o = out[:, :LOBES * 5].reshape(-1, LOBES, 5)
    mu, kappa, w = lobes(out)
    p = w * vmf_pdf(mu, kappa, wi)
    q = np.maximum(p.sum(axis=1), 1e-20)
    rr = p / q[:, None]
    pb = np.asarray(pb, np.float64)
    sg = 1 / (1 + np.exp(-out[:, 40]))
    csel = SEL_MIN + SEL_SPAN * sg
    qmix = np.maximum((1 - csel) * pb + csel * q, 1e-20)
    rho = (csel * q / qmix)[:, None]
    c = np.einsum("mkj,mj->mk", mu, wi)
    e2 = np.exp(-2 * kappa)
    dk = 1 / kappa - 2 * e2 / np.maximum(-np.expm1(-2 * kappa), 1e-20) + (c - 1)
    sig = 1 / (1 + np.exp(-o[:, :, 3]))
    sig = np.where(kappa >= KAPPA_MAX, 0.0, sig)
    ln = np.maximum(np.linalg.norm(o[:, :, :3], axis=2), 1e-12)
    dm = (wi[:, None, :] - mu * c[:, :, None]) * (kappa / ln)[:, :, None]
    g = np.zeros((out.shape[0], N_OUT_PAD))
    gv = g[:, :LOBES * 5].reshape(-1, LOBES, 5)
    ww = wgt[:, None]
    gv[:, :, 0:3] = -(ww * rho * rr)[:, :, None] * dm
    gv[:, :, 3] = -ww * rho * rr * dk * sig
    gv[:, :, 4] = -ww * rho * (rr - w)
    g[:, :LOBES * 5] = gv.reshape(-1, LOBES * 5)
    g[:, 40] = -wgt * (q - pb) * SEL_SPAN * sg * (1 - sg) / qmix
    if clamp is not None:
        g = np.clip(np.where(np.isfinite(g), g, 0.0), -clamp, clamp)
    active = wgt > 0
    g[~active] = 0.0
    deltas = [None] * 4
    deltas[3] = r(g)
    for l in (3, 2, 1):
        W = layers[l][0]
        back = deltas[l] @ r(W).T
        deltas[l - 1] = r(np.where(acts[l] > 0, back, 0.0))
    grads = []
    for l in range(4):
        dW = acts[l].T @ deltas[l]
        db = deltas[l].sum(axis=0)
        grads.append((dW, db))
    loss = float((wgt[active] * -np.log(qmix[active])).sum())
    return pack(grads), loss, float(wgt[active].sum())


def nll(params, enc, wi, weight, pb) -> float:
    out, _ = forward(params, enc, bf16_mode=False)
    q = mixture_pdf(out, wi)
    c = select_prob(out[:, 40])
    qmix = np.maximum((1 - c) * np.asarray(pb, np.float64) + c * q, 1e-20)
    return float((np.asarray(weight, np.float64) * -np.log(qmix)).sum())


def init_params(seed: int = 0, out_scale: float = 0.1) -> np.ndarray:
    """A random network in the flat layout (He-uniform, small output layer, zero padding)."""
    rng = np.random.default_rng(seed)
    layers = []
    for l, (k, n) in enumerate(SHAPES):
        bound = np.sqrt(6.0 / k) * (out_scale if l == 3 else 1.0)
        W = rng.uniform(-bound, bound, (k, n))
        b = rng.uniform(-0.1, 0.1, n)
        if l == 3:
            W[:, N_OUT:] = 0
            b[N_OUT:] = 0
        layers.append((W, b))
    return pack(layers)


def random_samples(m: int, seed: int = 1, lo=(-1, -1, -1), hi=(1, 1, 1)):
    """Seeded (x, n, wo, wi, w, p_bsdf) batch: positions in the box, unit directions, weights in
    (0, 4), BSDF densities in (0.05, 2)."""
    rng = np.random.default_rng(seed)
    lo, hi = np.asarray(lo, np.float64), np.asarray(hi, np.float64)
    x = lo + (hi - lo) * rng.random((m, 3))

    def unit(k):
        v = rng.normal(size=(k, 3))
        return v / np.linalg.norm(v, axis=1, keepdims=True)

    return x.astype(np.float32), unit(m).astype(np.float32), unit(m).astype(np.float32), unit(m).astype(np.float32), \
        (4 * rng.random(m)).astype(np.float32), (0.05 + 1.95 * rng.random(m)).astype(np.float32)


def finite_difference_check(seed: int = 0, m: int = 16, n_probe: int = 64, h: float = 1e-6) -> float:
    """Max relative error between the analytic FP64 gradient and central differences on n_probe
    random parameters (no BF16 rounding, no clamping)."""
    params = init_params(seed, out_scale=1.0)
    x, n, wo, wi, w, pb = random_samples(m, seed + 1)
    enc = encode(x, n, wo, (-1, -1, -1), (1, 1, 1))
    g, _, _ = nll_gradient(params, enc, wi, w, pb, bf16_mode=False, clamp=None)
    rng = np.random.default_rng(seed + 2)
    live = [i for i in range(N_PARAMS) if not _is_pad(i)]
    idx = rng.choice(live, n_probe, replace=False)
    worst = 0.0
    for i in idx:
        pp, pm = params.copy(), params.copy()
        pp[i] += h
        pm[i] -= h
        fd = (nll(pp, enc, wi, w, pb) - nll(pm, enc, wi, w, pb)) / (2 * h)
        worst = max(worst, abs(fd - g[i]) / max(1e-6, abs(fd), abs(g[i])))
    return worst


def _is_pad(i: int) -> bool:
    o = 0
    for l, (k, n) in enumerate(SHAPES):
        if i < o + k * n + n:
            if l != 3:
                return False
            rel = i - o
            col = rel % n if rel < k * n else rel - k * n
            return col >= N_OUT
        o += k * n + n
    return False
