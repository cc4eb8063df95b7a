"""What the trained surrogate gains over the method without it: on an unseen
microstructure, one call of the committed K = 50 network lands much closer
to the stencil's state after 50 steps than leaving the state unchanged (the
identity, i.e. surrogate + corrector with an untrained zero network) does,
field by field; over many calls etaL and c stay far closer than the
identity while etaS does not; and the surrogate + corrector stepper keeps
the solute mass on its initial value."""
import os

import numpy as np
import pytest

import phasefield_coarsening_gb300 as ppf
from phasefield_coarsening_gb300 import surrogate as S

pytestmark = pytest.mark.gpu

WEIGHTS_DIR = os.path.join(os.path.dirname(ppf.__file__), "weights")
WEIGHTS = os.path.join(WEIGHTS_DIR, "surrogate_w16_k50.npz")
# both K = 50 networks: the configured width 32 and the cheaper width 16
K50 = ["surrogate_w32_k50.npz", "surrogate_w16_k50.npz"]


def sim_of(shape, state):
    s = ppf.Simulation(shape, ppf.params_default(dt=S.DT), "periodic", "f32")
    s.upload(*state)
    return s


@pytest.mark.parametrize("weights", K50)
def test_trained_network_beats_the_identity(weights):
    net = S.load(os.path.join(WEIGHTS_DIR, weights), gain=(1.0, 1.0, 1.0))   # the raw network, one call
    k = net.config["k_steps"]
    scale = np.asarray(net.config["out_scale"])
    shape = (32, 128, 128)
    a = sim_of(shape, S.microstructure(shape, seed=424242, vf=0.25))
    a.step(300)                                  # relaxed interfaces, as in training
    b = sim_of(shape, a.download())
    b.step(k)                                    # the stencil's answer
    c = sim_of(shape, a.download())
    net.advance(c, 1)                            # the network's answer
    x, y, z = a.download(), b.download(), c.download()
    e_id = [float(np.mean(((q - p) / sc) ** 2)) for p, q, sc in zip(x, y, scale)]
    e_net = [float(np.mean(((q - r) / sc) ** 2)) for q, r, sc in zip(y, z, scale)]
    for s in (a, b, c):
        s.close()
    net.close()
    # one call, normalised squared error against no change: etaL and c at
    # least 2x closer; etaS, which moves ~9x less per call, clearly closer too
    # (the width-32 network: 0.51 of the identity's error)
    for name, n, i, bound in zip(("etaS", "etaL", "c"), e_net, e_id, (0.6, 0.5, 0.5)):
        assert n < bound * i, (name, n, i)


@pytest.mark.parametrize("weights", K50)
def test_many_cycles_per_field_against_the_identity(weights):
    """Four stepper cycles (10 calls of K = 50 + 50 corrector steps each) on
    an unseen microstructure, per field ||surrogate - stencil|| /
    ||stencil - start|| against the same schedule with the calls replaced by
    the identity.  etaL and c: the network carries most of the change.
    etaS: the per-call errors add up over many calls of a relaxed state, and
    the result stays slightly farther from the stencil than leaving etaS
    unchanged (measured 1.05x the identity's error for the width-32 network
    with its stored etaS gain, 1.14x for width 16); no etaS gain from 0.01 to
    1 on other held-out rollouts brought it below the identity
    (surrogate.calibrate_gain), so the bound records that finding."""
    net = S.load(os.path.join(WEIGHTS_DIR, weights))
    shape = (32, 128, 128)
    state = S.microstructure(shape, seed=515151, vf=0.25)
    r = S.compare_to_stencil(net, state, cycles=4, calls=10, corrector_steps=50, warmup=500)
    net.close()
    f = r["field_err_vs_change"]
    print(f)
    assert f["surrogate"]["etaL"] < 0.6 * f["identity"]["etaL"]
    assert f["surrogate"]["c"] < 0.6 * f["identity"]["c"]
    assert f["surrogate"]["etaS"] < 1.25 * f["identity"]["etaS"]
    assert r["mass_drift"] <= 1e-12 and r["fallbacks"] == 0


def test_stepper_conserves_mass_and_counts_steps():
    net = S.load(WEIGHTS)
    shape = (32, 64, 128)
    sim = sim_of(shape, S.microstructure(shape, seed=77, vf=0.3))
    sim.step(300)
    m0 = sim.reduce()["mass"]
    st = S.Stepper(net, sim, calls=4, corrector_steps=20)
    n = st.cycle() + st.cycle()
    r = sim.reduce()
    assert n == 2 * (4 * net.config["k_steps"] + 20)
    assert r["steps"] == 300 + n
    assert abs(r["mass"] / m0 - 1.0) < 1e-12
    assert r["nonfinite"] == 0
    st.close()
    sim.close()
    net.close()
