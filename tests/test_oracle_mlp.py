"""The learned rectifier's CPU restatement (oracle/mlp_oracle.py) on its own:
its analytic gradients against central differences of its loss, and its
feature and fallback definitions.  No GPU."""
import numpy as np

import mlp_oracle as M


def synthetic_records(n, seed=0):
    rng = np.random.default_rng(seed)
    mean = rng.uniform(0.1, 2.0, (n, 3)) * np.array([1.0, 0.3, 0.3])
    sigma = rng.uniform(0.01, 0.5, (n, 3))
    hist = mean + rng.normal(0, 1.5, (n, 3)) * sigma          # some inside the box, some clipped
    cur = mean + rng.normal(0, 1.0, (n, 3)) * sigma
    truth = rng.uniform(0.0, 2.0, (n, 3))
    f = M.features(mean, sigma, mean - sigma, mean + sigma, hist, cur, rng.uniform(0, 20, n), rng.normal(0, 1, n),
                   np.zeros(n))
    flags = (rng.uniform(size=n) < 0.1).astype(np.uint32)   # a tenth with a fixed blend weight
    return dict(features=M.half(f), mean=mean, sigma=sigma, history=hist, current=cur, truth=truth,
                gamma=np.full(n, 1.0), alpha_fixed=np.where(flags == 1, 1.0, 0.1), flags=flags)


def weights(seed=0, o1_bias=0.0):
    rng = np.random.default_rng(seed)
    w = dict(w1=rng.uniform(-0.3, 0.3, (32, 32)), b1=rng.uniform(-0.1, 0.1, 32), w2=rng.uniform(-0.3, 0.3, (32, 32)),
             b2=rng.uniform(-0.1, 0.1, 32), w3=rng.uniform(-0.2, 0.2, (2, 32)), b3=np.array([-2.0, o1_bias]))
    for k in ("w1", "w2"):
        w[k][31, :] = 0.0
        w[k][:, 31] = 0.0
    w["w3"][:, 31] = 0.0
    w["b1"][31] = w["b2"][31] = 0.0
    return w


def numeric_grad(w, rec, key, idx, h=1e-6):
    wp = {k: np.array(v, copy=True) for k, v in w.items()}
    wm = {k: np.array(v, copy=True) for k, v in w.items()}
    wp[key][idx] += h
    wm[key][idx] -= h
    return (M.loss_exact(wp, rec) - M.loss_exact(wm, rec)) / (2 * h)


def test_analytic_gradients_match_central_differences():
    rec = synthetic_records(64)
    for o1_bias in (0.0, 1.6):   # box scales inside [0.5, 2], and partly outside (fallback and penalty)
        w = weights(1, o1_bias)
        _, g = M.gradients_exact(w, rec)
        rng = np.random.default_rng(2)
        for key, shape in (("w1", (32, 32)), ("w2", (32, 32)), ("w3", (2, 32)), ("b1", (32,)), ("b2", (32,)),
                           ("b3", (2,))):
            for _ in range(6):
                idx = tuple(int(rng.integers(0, s)) for s in shape)
                if (key in ("w1", "w2") and (idx[0] == 31 or idx[1] == 31)) or (key == "w3" and idx[1] == 31) or \
                        (key in ("b1", "b2") and idx[0] == 31):
                    assert g[key][idx] == 0.0  # the constant unit carries no weight
                    continue
                num = numeric_grad(w, rec, key, idx)
                assert abs(num - g[key][idx]) <= 1e-5 * max(1.0, abs(num)), (o1_bias, key, idx, num, g[key][idx])


def test_scale_outside_range_falls_back_to_plain_clip():
    rec = synthetic_records(16, seed=3)
    rec["flags"][:] = 0
    rec["alpha_fixed"][:] = 0.1  # the plain alpha the fallback blends with
    o = np.zeros((16, 2))
    o[:, 1] = 3.0  # box scale 8: outside [0.5, 2]
    loss_out, d = M.loss_and_output_grad(rec, o)
    o_plain = np.zeros((16, 2))
    o_plain[:, 0] = np.log(0.1 / 0.9)  # the plain alpha 0.1, scale 1
    loss_plain, _ = M.loss_and_output_grad(rec, o_plain)
    # the plain result plus the penalty (3 - 1)^2 per record, and no gradient for alpha
    np.testing.assert_allclose(loss_out, loss_plain + M.PENALTY * 4.0, rtol=1e-9)
    assert np.all(d[:, 0] == 0.0) and np.all(d[:, 1] > 0.0)


def test_features_scale_invariant():
    rng = np.random.default_rng(4)
    mean = rng.uniform(0.5, 2, (8, 3))
    sigma = rng.uniform(0.01, 0.3, (8, 3))
    hist, cur = mean + sigma, mean - 0.5 * sigma
    f1 = M.features(mean, sigma, mean - sigma, mean + sigma, hist, cur, 1.0, 0.0, 0.0)
    assert f1.shape == (8, 32) and np.all(f1[:, 31] == 1.0)
    # deviation features are in units of sigma: hist = mean + sigma gives about 1/4
    np.testing.assert_allclose(f1[:, 18:21], 0.25, atol=0.01)


def test_outlier_current_sample_caps_the_blend_weight():
    """A current sample farther from the box mean (luma) than twice the plain box's half
    extent: the network's blend weight is held to the plain one and passes no gradient;
    just inside that distance it is the network's own."""
    n = 4
    mean = np.tile([1.0, 0.0, 0.0], (n, 1))
    sigma = np.full((n, 3), 0.2)
    cur = mean.copy()
    cur[:, 0] += np.array([0.5, 0.39, -0.45, 0.5])   # 2.5, 1.95, 2.25 and 2.5 sigma from the mean
    rec = dict(mean=mean, sigma=sigma, history=mean + 0.05, current=cur, truth=cur.copy(), gamma=np.full(n, 1.0),
               alpha_fixed=np.full(n, 0.1), flags=np.zeros(n, dtype=np.uint32))
    o = np.zeros((n, 2))
    o[:, 0] = [2.0, 2.0, 2.0, -4.0]   # network weights 0.88, 0.88, 0.88 and 0.018
    loss, d = M.loss_and_output_grad(rec, o)
    loss_plain, _ = M.loss_and_output_grad(rec, np.where(np.arange(2) == 0, np.log(0.1 / 0.9), 0.0) * np.ones((n, 2)))
    assert d[0, 0] == 0.0 and d[2, 0] == 0.0           # capped: the plain weight, no gradient
    assert abs(loss[0] - loss_plain[0]) < 1e-12 and abs(loss[2] - loss_plain[2]) < 1e-12
    assert d[1, 0] != 0.0                               # inside 2 sigma: the network's weight
    assert d[3, 0] != 0.0                               # below the plain weight: not capped
