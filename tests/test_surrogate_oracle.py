"""The CPU restatement of the surrogate network (oracle/surrogate_ref.py):
its backward pass against finite differences of its own forward pass in
float64, and its BF16 rounding against torch's."""
import numpy as np
import pytest

from oracle import surrogate_ref as sr

CFG = {"width": 16, "c_solid": 0.47603, "c_liquid": 0.99903, "in_scale_c": 1000.0,
       "out_scale": [1e-2, 1e-2, 1e-3], "loss_weight": [1.0, 0.5, 2.0]}


def smooth_state(shape, seed):
    rng = np.random.default_rng(seed)
    z, y, x = np.meshgrid(*[np.arange(n) for n in shape], indexing="ij")
    ph = rng.uniform(0, 2 * np.pi, 3)
    eS = 0.5 + 0.45 * np.sin(2 * np.pi * x / shape[2] + ph[0]) * np.cos(2 * np.pi * y / shape[1] + ph[1])
    eS = np.clip(eS + 0.02 * rng.standard_normal(shape), 0.0, 1.0)
    eL = np.clip(1.0 - eS + 0.01 * rng.standard_normal(shape), 0.0, 1.0)
    h = eS ** 2 / (eS ** 2 + eL ** 2)
    c = h * CFG["c_solid"] + (1 - h) * CFG["c_liquid"] + 1e-3 * rng.uniform(-1, 1, shape)
    return eS, eL, c


def test_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    a = np.concatenate([rng.standard_normal(10000) * 10.0 ** rng.integers(-8, 8, 10000),
                        [0.0, -0.0, 1.0, 1.00390625, 1.005859375, 65504.0, 3.0e38]]).astype(np.float32)
    ref = torch.from_numpy(a).to(torch.bfloat16).to(torch.float64).numpy()
    assert np.array_equal(sr.bf16(a), ref)


def test_backward_matches_finite_differences():
    shape = (3, 4, 5)
    state = smooth_state(shape, 1)
    target = tuple(np.asarray(s, np.float32) + np.float32(d) * np.random.default_rng(2).standard_normal(shape)
                   for s, d in zip(state, (1e-2, 1e-2, 1e-3)))
    params = sr.init_params(16, seed=3, last_scale=0.5).astype(np.float64)
    params += 0.01 * np.random.default_rng(4).standard_normal(params.size)
    loss, g = sr.loss_and_grad(state, target, params, CFG, rounding=None)
    assert loss > 0
    rng = np.random.default_rng(5)
    # weights of every layer, biases of the output and of a hidden layer
    idx = []
    off = 0
    for li, (ci, co) in enumerate(sr.layer_channels(16)):
        n = 27 * co * ci
        W = np.arange(off, off + n).reshape(27, co, ci)
        used_ci = sr.N_FEATURES if li == 0 else ci
        used_co = 3 if li == sr.LAYERS - 1 else co
        idx += list(rng.choice(W[:, :used_co, :used_ci].ravel(), 4, replace=False))
        off += n
        idx += list(range(off, off + min(used_co, 2)))
        off += co
    for i in idx:
        h = 1e-6 * max(1.0, abs(params[i]))
        p1, p2 = params.copy(), params.copy()
        p1[i] += h
        p2[i] -= h
        fd = (sr.loss_and_grad(state, target, p1, CFG, rounding=None)[0] -
              sr.loss_and_grad(state, target, p2, CFG, rounding=None)[0]) / (2 * h)
        assert abs(fd - g[i]) <= 1e-5 * abs(g).max() + 1e-4 * abs(fd), (i, fd, g[i])


def test_flatten_roundtrip_and_zero_padding():
    p = sr.init_params(32, seed=0, last_scale=1.0)
    layers = sr.unflatten(p, 32)
    assert np.array_equal(sr.flatten(layers).astype(np.float32), p)
    W0, _ = layers[0]
    assert not W0[:, :, sr.N_FEATURES:].any()          # padded input channels
    W5, b5 = layers[-1]
    assert not W5[:, 3:, :].any() and not b5.any()


def test_features_carry_what_bf16_drops():
    rng = np.random.default_rng(3)
    eS = rng.random((2, 3, 4)).astype(np.float32)
    eL = (1 - eS).astype(np.float32)
    c = np.full(eS.shape, 0.9, np.float32)
    f = sr.features(eS, eL, c, CFG)
    # hi + lo reconstructs the FP32 field to far better than BF16 alone
    for k, x in ((3, eS), (4, eL)):
        rec = sr.bf16(x) + sr.bf16(f[k]) / 256.0
        assert np.abs(rec - x).max() < 2.0 ** -16 * 1.01
        assert np.abs(sr.bf16(x) - x).max() > 2.0 ** -14
