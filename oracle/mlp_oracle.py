"""CPU restatement of the learned rectifier (test infrastructure only).

The learned form has no counterpart in the reference; this module is its
definition in FP64 numpy, used by the tests as the checker of the library's
tensor-core kernels (taa-star_gb300/csrc/learned.cu, learned.cuh):

* ``features`` - the 32 network inputs from a pixel's box, history and
  current colour (learned.cuh ``features``);
* ``forward`` / ``gradients`` - the network (32 -> 32 -> 32 -> 2, ReLU) and
  the gradient of the training loss with respect to every weight, rounding to
  FP16 at the points where the kernels hand FP16 operands to the tensor cores
  (weights, inputs, activations, back-propagated gradients), so the sums can
  be compared tightly with the kernels' FP32 accumulation;
* ``loss_and_output_grad`` - the loss of one record (its rectified, blended
  RGB against the ground truth, squared, in linear space as the library is
  built by default) and its derivative with respect to the two network
  outputs (learned.cu ``record_loss``);
* ``gradients_exact`` - the same gradients without any FP16 rounding, which
  the tests hold against central differences.
"""
from __future__ import annotations

import numpy as np

LN2 = 0.69314718055994531
PENALTY = 1.0  # weight of the pull on a log2 box scale outside [-1, 1] (learned.cu kPenalty)
OUTLIER_K = 2.0  # a current sample beyond K * gamma * sigma of the box mean caps the blend weight (learned.cuh)


def half(x):
    return np.asarray(x, dtype=np.float64).astype(np.float16).astype(np.float64)


def features(mean, sigma, mn, mx, hist, cur, vel_px, depth_rel, rejected):
    """The 32 inputs of one or many pixels (arrays [..., 3] in YCoCg)."""
    mean, sigma, mn, mx, hist, cur = (np.asarray(a, np.float64) for a in (mean, sigma, mn, mx, hist, cur))
    inv = 1.0 / (np.maximum(mean[..., 0], 0.0) + 0.05)
    f = np.zeros(mean.shape[:-1] + (32,))
    i3 = inv[..., None]
    f[..., 0:3] = mean * i3
    f[..., 3:6] = sigma * i3
    f[..., 6:9] = mn * i3
    f[..., 9:12] = mx * i3
    f[..., 12:15] = hist * i3
    f[..., 15:18] = cur * i3
    dev = (hist - mean) / (sigma + 1e-3 / i3)
    f[..., 18:21] = np.clip(dev, -8, 8) * 0.25
    f[..., 21] = np.minimum(vel_px, 64.0) / 16.0
    f[..., 22] = np.clip(depth_rel, -8, 8) * 0.125
    f[..., 23] = np.asarray(rejected, np.float64)
    ma = np.max(np.abs(hist - mean) / (sigma + 1e-7), axis=-1)
    f[..., 24] = np.minimum(ma, 8.0) * 0.125
    f[..., 25] = np.log2(np.maximum(mean[..., 0], 0.0) + 1e-3) * 0.125
    f[..., 26] = (mx[..., 0] - mn[..., 0]) * inv
    f[..., 27:30] = (cur - mean) * i3
    f[..., 30] = (hist[..., 0] - cur[..., 0]) * inv
    f[..., 31] = 1.0
    return np.clip(f, -60000.0, 60000.0)


CONST = 31  # input 31 and hidden unit 31 of each layer are the constant 1


def effective(w):
    """The matrices the kernels multiply by: biases in column 31, the constant
    unit in row 31 of layers 1 and 2 (learned.cu eff1, eff2, eff3)."""
    e1 = np.array(w["w1"], np.float64).reshape(32, 32).copy()
    e2 = np.array(w["w2"], np.float64).reshape(32, 32).copy()
    e3 = np.array(w["w3"], np.float64).reshape(2, 32).copy()
    e1[:, CONST] = w["b1"]
    e2[:, CONST] = w["b2"]
    e3[:, CONST] = w["b3"]
    for e in (e1, e2):
        e[CONST, :] = 0.0
        e[CONST, CONST] = 1.0
    return dict(w1=e1, w2=e2, w3=e3)


def forward(w, f, rounded=True):
    """Outputs [n, 2] and the activations the backward pass needs."""
    r = half if rounded else (lambda a: np.asarray(a, np.float64))
    q = {k: r(v) for k, v in effective(w).items()}
    x = r(f)
    h1 = np.maximum(r(x @ q["w1"].T), 0.0)
    h2 = np.maximum(r(h1 @ q["w2"].T), 0.0)
    o = h2 @ q["w3"].T
    return o, dict(x=x, h1=h1, h2=h2, q=q)


def _g(x):
    return np.asarray(x, np.float64)


def _dg(x):
    return np.ones_like(np.asarray(x, np.float64))


def loss_and_output_grad(rec, o):
    """Loss per record and d loss / d outputs [n, 2] (learned.cu record_loss)."""
    o0, o1 = o[:, 0], o[:, 1]
    fixed = (rec["flags"] & 1) != 0
    s = np.exp2(o1)
    s_in = (s >= 0.5) & (s <= 2.0)
    mean, sigma, hist, cur, gt = rec["mean"], rec["sigma"], rec["history"], rec["current"], rec["truth"]
    a_net = 1.0 / (1.0 + np.exp(-o0))
    # a current sample farther from the box mean in luma than twice gamma * sigma: the blend
    # weight no more than the plain one (learned.cuh current_outlier)
    outlier = np.abs(cur[:, 0] - mean[:, 0]) > OUTLIER_K * rec["gamma"] * sigma[:, 0] + 1e-7
    capped = ~fixed & s_in & outlier & (a_net > rec["alpha_fixed"])
    alpha = np.where(fixed | ~s_in | capped, rec["alpha_fixed"], a_net)
    sc = np.where(s_in, s, 1.0)
    g = rec["gamma"][:, None]
    e = sc[:, None] * g * sigma + 1e-7
    d = hist - mean
    q = np.abs(d / e)
    k = np.argmax(q, axis=1)
    ma = q[np.arange(len(k)), k]
    clipped = ma > 1.0
    kf = np.where(clipped, 1.0 / np.where(clipped, ma, 1.0), 1.0)
    hc = mean + d * kf[:, None]
    out = hc * (1.0 - alpha[:, None]) + cur * alpha[:, None]
    tmp = out[:, 0] - out[:, 2]
    rgb = np.stack([tmp + out[:, 1], out[:, 0] + out[:, 2], tmp - out[:, 1]], axis=1)
    diff = _g(rgb) - _g(gt)
    loss = np.sum(diff * diff, axis=1)
    dr = 2.0 * diff * _dg(rgb)
    dout = np.stack([dr[:, 0] + dr[:, 1] + dr[:, 2], dr[:, 0] - dr[:, 2], -dr[:, 0] + dr[:, 1] - dr[:, 2]], axis=1)
    dalpha = np.sum(dout * (cur - hc), axis=1)
    dk = np.abs(d[np.arange(len(k)), k])
    sk = sigma[np.arange(len(k)), k]
    dsc = np.where(clipped, np.sum(dout * (1.0 - alpha[:, None]) * d, axis=1) * (rec["gamma"] * sk /
                                                                                   np.where(clipped, dk, 1.0)), 0.0)
    d0 = np.where(fixed | ~s_in | capped, 0.0, dalpha * alpha * (1.0 - alpha))
    d1 = np.where(s_in, dsc * s * LN2, 0.0)
    # outside the trusted scale range: the plain result and a penalty pulling o1 back
    over = np.abs(o1) - 1.0
    loss = loss + np.where(s_in, 0.0, PENALTY * over * over)
    d1 = np.where(s_in, d1, 2.0 * PENALTY * over * np.sign(o1))
    return loss, np.stack([d0, d1], axis=1)


def gradients(w, rec, rounded=True):
    """Loss sum and gradient sums (dict like the weights) over the records."""
    r = half if rounded else (lambda a: np.asarray(a, np.float64))
    o, act = forward(w, rec["features"], rounded)
    loss, do = loss_and_output_grad(rec, o)
    do = r(do)
    q, x, h1, h2 = act["q"], act["x"], act["h1"], act["h2"]
    g2 = np.where(h2 > 0, r(do @ q["w3"]), 0.0)
    g1 = np.where(h1 > 0, r(g2 @ q["w2"]), 0.0)
    d1, d2, d3 = g1.T @ x, g2.T @ h1, do.T @ h2
    # gradients of the effective matrices -> of the masters (learned.cu map_grads)
    grad = dict(b1=d1[:, CONST].copy(), b2=d2[:, CONST].copy(), b3=d3[:, CONST].copy())
    grad["b1"][CONST] = 0.0
    grad["b2"][CONST] = 0.0
    for k, d in (("w1", d1), ("w2", d2), ("w3", d3)):
        d = d.copy()
        d[:, CONST] = 0.0
        if k != "w3":
            d[CONST, :] = 0.0
        grad[k] = d
    return float(loss.sum()), grad


def gradients_exact(w, rec):
    return gradients(w, rec, rounded=False)


def loss_exact(w, rec):
    o, _ = forward(w, rec["features"], rounded=False)
    return float(loss_and_output_grad(rec, o)[0].sum())
