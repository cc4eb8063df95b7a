"""The surrogate on the GPU (tcgen05 BF16 implicit-GEMM convolutions) against
the CPU restatement oracle/surrogate_ref.py: network output, loss and the
gradient of every parameter; the FP64 solute-mass projection; the
surrogate as a time stepper; training on stencil trajectories."""
import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state
from oracle import surrogate_ref as sr

pytestmark = pytest.mark.gpu

DT = 0.8 / (6.0 * 1e-14)
ULP = 2.0 ** -24


def make_sim(shape, state, bc="periodic"):
    s = ppf.Simulation(shape, ppf.params_default(dt=DT), bc=bc, precision="f32")
    s.upload(*state)
    return s


def perturbed(state, seed, amp=(5e-3, 5e-3, 5e-4)):
    rng = np.random.default_rng(seed)
    return tuple(a + d * rng.standard_normal(a.shape) for a, d in zip(state, amp))


# tolerances: the device accumulates in FP32 in another order than the
# oracle's FP64, which moves an occasional BF16 rounding of an activation by
# one BF16 ulp (2^-8 relative); the effect on outputs and gradients stays at
# the 1e-3 level in the L2 norm
@pytest.mark.parametrize("width,shape", [(32, (6, 5, 128)), (16, (4, 9, 256)), (32, (3, 3, 128))])
def test_forward_matches_oracle(width, shape):
    state = smooth_state(shape, seed=11)
    p = sr.init_params(width, seed=7, last_scale=1.0)
    with ppf.Surrogate(width=width) as net, make_sim(shape, state) as sim:
        net.set_params(p)
        got = net.predict(sim)
        cfg = net.config
    pred, _ = sr.forward(state, p, cfg)
    ref = pred * np.asarray(cfg["out_scale"])[:, None, None, None]
    assert np.abs(got - ref).max() <= 2e-2 * np.abs(ref).max()
    assert np.linalg.norm(got - ref) <= 5e-3 * np.linalg.norm(ref)


@pytest.mark.parametrize("width", [16, 32])
def test_forward_on_noflux_domain_matches_oracle(width):
    """Inference on a no-flux domain: every activation's halo holds the
    mirror images (ghost -1 = cell 0, ghost n = cell n-1)."""
    shape = (5, 6, 128)
    state = smooth_state(shape, seed=17)
    p = sr.init_params(width, seed=8, last_scale=1.0)
    with ppf.Surrogate(width=width) as net, make_sim(shape, state, bc="noflux") as sim:
        net.set_params(p)
        got = net.predict(sim)
        cfg = net.config
    pred, _ = sr.forward(state, p, cfg, bc="noflux")
    ref = pred * np.asarray(cfg["out_scale"])[:, None, None, None]
    assert np.abs(got - ref).max() <= 2e-2 * np.abs(ref).max()
    assert np.linalg.norm(got - ref) <= 5e-3 * np.linalg.norm(ref)
    # and it is not the periodic answer
    per, _ = sr.forward(state, p, cfg)
    per = per * np.asarray(cfg["out_scale"])[:, None, None, None]
    assert np.linalg.norm(per - ref) > 20 * np.linalg.norm(got - ref)


@pytest.mark.parametrize("width", [32, 16])
def test_loss_and_gradients_match_oracle(width):
    shape = (4, 6, 128)
    s0 = smooth_state(shape, seed=21)
    s1 = perturbed(s0, 22)
    p = sr.init_params(width, seed=5, last_scale=1.0)
    with ppf.Surrogate(width=width, loss_weight=(1.0, 0.5, 2.0)) as net, \
            make_sim(shape, s0) as a, make_sim(shape, s1) as b:
        net.set_params(p)
        loss, g = net.loss_grad(a, b)
        loss2, g2 = net.loss_grad(a, b)
        cfg = net.config
    assert loss == loss2 and np.array_equal(g, g2)        # deterministic
    rl, rg = sr.loss_and_grad(s0, s1, p, cfg)
    assert abs(loss - rl) <= 1e-3 * rl
    off = 0
    for li, (ci, co) in enumerate(sr.layer_channels(width)):
        for n, what in ((27 * co * ci, "W"), (co, "b")):
            seg = slice(off, off + n)
            off += n
            ref = rg[seg]
            assert np.linalg.norm(g[seg] - ref) <= 2e-2 * np.linalg.norm(ref) + 1e-12, (li, what)
    assert off == g.size


def test_mass_projection_lands_on_target():
    shape = (24, 20, 36)
    with make_sim(shape, smooth_state(shape, seed=3)) as s:
        m0 = s.reduce()["mass"]
        s.step(300)
        eS0, eL0, c0 = s.download()
        s.mass_project(m0)                  # undo the FP32 drift of 300 steps
        assert abs(s.reduce()["mass"] - m0) <= 4 * ULP
        drift = abs(c0.sum() - m0)
        assert np.abs(s.download()[2] - c0).max() <= (np.ceil(drift / (c0.size * ULP)) + 2) * ULP
        for target in (m0 + 0.37, m0 - 1.5e-3):
            s.mass_project(target)
            m = s.reduce()["mass"]
            assert abs(m - target) <= 4 * ULP, (m - target)
        eS1, eL1, c1 = s.download()
        assert np.array_equal(eS0, eS1) and np.array_equal(eL0, eL1)
        s.step(5)                       # ghosts stayed consistent: a step still matches a fresh upload
        ref = make_sim(shape, (eS1, eL1, c1))
        ref.step(5)
        for a, b in zip(s.download(), ref.download()):
            assert np.array_equal(a, b)
        ref.close()


def test_advance_is_predict_plus_projection():
    shape = (6, 7, 128)
    state = smooth_state(shape, seed=4)
    p = sr.init_params(32, seed=9, last_scale=0.3)
    with ppf.Surrogate(width=32, k_steps=50) as net, make_sim(shape, state) as sim:
        net.set_params(p)
        s32 = [np.asarray(a, np.float32).astype(np.float64) for a in sim.download()]
        m0 = sim.reduce()["mass"]
        d = net.predict(sim)
        net.advance(sim, 1)
        st = sim.reduce()
        eS, eL, c = sim.download()
    assert st["steps"] == 50
    assert abs(st["mass"] - m0) <= 4 * ULP
    for got, base, dd in ((eS, s32[0], d[0]), (eL, s32[1], d[1])):
        ref = (base.astype(np.float32) + dd.astype(np.float32)).astype(np.float64)
        assert np.abs(got - ref).max() <= 2.5e-7 * np.abs(ref).max()
    # c: the prediction, then a near-uniform shift that restores sum(c)
    ref_c = s32[2] + d[2]
    ref_c += (m0 - ref_c.sum()) / ref_c.size
    assert np.abs(c - ref_c).max() <= 4e-7


def test_zero_output_layer_is_the_identity():
    shape = (5, 5, 128)
    state = smooth_state(shape, seed=8)
    with ppf.Surrogate(width=16) as net, make_sim(shape, state) as sim:
        net.set_params(sr.init_params(16, seed=1, last_scale=0.0))
        before = sim.download()
        net.advance(sim, 3)
        after = sim.download()
    for a, b in zip(before, after):
        assert np.array_equal(a, b)


def test_training_on_stencil_pairs_reduces_the_loss():
    from phasefield_coarsening_gb300 import ic
    shape = (24, 32, 128)
    eS, eL, c, _ = ic.generate(shape, radius=("uniform", 3.0, 6.0), count=24, seed=2)
    k = 20
    with make_sim(shape, (eS, eL, c)) as a, make_sim(shape, (eS, eL, c)) as b:
        a.step(40)
        b.copy_from(a)
        b.step(k)
        x = [np.asarray(v) for v in a.download()]
        y = [np.asarray(v) for v in b.download()]
        rms = [float(np.sqrt(np.mean((q - r) ** 2))) for q, r in zip(y, x)]
        with ppf.Surrogate(width=32, k_steps=k, out_scale=rms) as net:
            net.set_params(sr.init_params(32, seed=0, last_scale=0.0))
            first = net.loss_grad(a, b)[0]
            for _ in range(400):
                net.train_step(a, b, lr=1e-3, want_loss=False)
            final = net.loss_grad(a, b)[0]
    assert 0.2 < first < 2.0          # zero prediction: loss = mean of squared normalised targets
    assert final < 0.3 * first, (first, final)
