"""The surrogate + corrector stepper's decisions (host logic, no GPU): a
cycle advances calls x k + corrector steps, ends on the initial solute mass,
and is redone by the stencil alone from its snapshot when the result has
non-finite cells, a rising free energy or a drifting solid fraction."""
import math

import pytest

from phasefield_coarsening_gb300 import surrogate as S


class FakeSim:
    def __init__(self, stats_after):
        self.log = []
        self.state = "s0"
        self.stats = [{"mass": 10.0, "free_energy": 100.0, "solid": 50.0, "nonfinite": 0}]
        self.stats_after = stats_after
        self.shape, self.params, self.bc = (4, 4, 128), None, 0

    def reduce(self):
        return dict(self.stats[-1])

    def copy_from(self, other):
        self.log.append(("copy_from", other.state))
        self.state = other.state

    def step(self, n):
        self.log.append(("step", n))
        if self.stats_after:
            self.stats.append(self.stats_after.pop(0))

    def mass_project(self, m):
        self.log.append(("mass_project", m))


class FakeSnap:
    def __init__(self):
        self.state = None

    def copy_from(self, other):
        self.state = other.state


class FakeNet:
    config = {"k_steps": 50}

    def __init__(self, sim):
        self.sim = sim

    def advance(self, sim, calls):
        sim.log.append(("advance", calls))
        sim.state = "surrogate"


def run_cycle(after):
    sim = FakeSim([after])
    st = S.Stepper(FakeNet(sim), sim, calls=10, corrector_steps=50, snapshot=FakeSnap())
    n = st.cycle()
    return st, sim, n


def test_good_cycle_keeps_the_surrogate_result():
    st, sim, n = run_cycle({"mass": 10.0, "free_energy": 99.9, "solid": 50.1, "nonfinite": 0})
    assert n == 10 * 50 + 50 and st.fallbacks == 0
    assert sim.log == [("advance", 10), ("step", 50), ("mass_project", 10.0)]


@pytest.mark.parametrize("bad", [
    {"mass": 10.0, "free_energy": 100.1, "solid": 50.0, "nonfinite": 0},       # free energy rose
    {"mass": 10.0, "free_energy": 99.0, "solid": 49.0, "nonfinite": 0},        # solid fraction moved 2 %
    {"mass": 10.0, "free_energy": 99.0, "solid": 50.0, "nonfinite": 3},        # non-finite cells
    {"mass": 10.0, "free_energy": math.nan, "solid": 50.0, "nonfinite": 0},    # non-finite energy
])
def test_bad_cycle_falls_back_to_the_stencil(bad):
    st, sim, n = run_cycle(bad)
    assert st.fallbacks == 1 and n == 550
    # restored from the snapshot taken before the surrogate calls, then the stencil alone
    assert sim.log[:2] == [("advance", 10), ("step", 50)]
    assert sim.log[2] == ("copy_from", "s0")
    assert sim.log[3] == ("step", 550)
    assert sim.log[4] == ("mass_project", 10.0)


def test_unchecked_stepper_never_falls_back():
    sim = FakeSim([{"mass": 10.0, "free_energy": 500.0, "solid": 1.0, "nonfinite": 9}])
    st = S.Stepper(FakeNet(sim), sim, calls=2, corrector_steps=5, check=False)
    assert st.cycle() == 105 and st.fallbacks == 0


def test_init_params_match_the_documented_layout():
    p = S.init_params(16, seed=0)
    assert p.size == 6 * (27 * 16 * 16 + 16)
    last = p[-(27 * 16 * 16 + 16):]
    assert not last.any()            # output layer starts at zero: the identity map
