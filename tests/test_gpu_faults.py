"""Failure detection without a GPU fault: the step kernel's device waits are
bounded; a test hook makes one wait per CTA run out, the host reads the
error status, and the context stays usable."""
import numpy as np
import pytest

import oracle
import phasefield_coarsening_gb300 as ppf
from helpers import smooth_state

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["f64", "f32"])
def test_wait_limit_expiry_is_reported_and_context_recovers(precision):
    shape = (20, 30, 70)
    st = smooth_state(shape, seed=4)
    with ppf.Simulation(shape, precision=precision) as s:
        s.upload(*st)
        s.set_wait_limit(0.05)
        s.debug_inject(ppf.INJECT_STALL_WAIT)
        s.step(1)
        with pytest.raises(ppf.PPFError) as e:
            s.sync()
        assert e.value.code == -6
        s.sync()                      # the error word was read and cleared
        s.set_wait_limit(1.0)
        s.upload(*st)
        s.step(5)
        out = s.download()
    ref = oracle.run(*st, 5, bc=0)
    tol = 1e-12 if precision == "f64" else 1e-5
    assert max(float(np.abs(a - b).max()) for a, b in zip(out, ref[:3])) <= tol


def test_wait_limit_validation():
    with ppf.Simulation((4, 4, 4)) as s:
        with pytest.raises(ppf.PPFError):
            s.set_wait_limit(0.0)
        with pytest.raises(ppf.PPFError):
            s.debug_inject(99)


def test_surrogate_wait_limit_expiry_is_reported_and_recovers():
    """The same for the tensor-core convolution: one input row's copies never
    complete, the bounded waits run out, every role drains and exits, the
    host sees PPF_ETIMEOUT, and the next call is exact again."""
    from oracle import surrogate_ref as sr
    shape = (6, 5, 128)
    st = smooth_state(shape, seed=9)
    p = sr.init_params(16, seed=2, last_scale=0.3)
    with ppf.Surrogate(width=16) as net, ppf.Simulation(shape, bc="periodic", precision="f32") as s:
        net.set_params(p)
        s.upload(*st)
        s.set_wait_limit(0.05)
        net.debug_inject(ppf.INJECT_STALL_WAIT)
        net.advance(s, 1)
        with pytest.raises(ppf.PPFError) as e:
            s.sync()
        assert e.value.code == -6
        s.set_wait_limit(1.0)
        s.upload(*st)
        net.advance(s, 1)
        got = s.download()
    with ppf.Surrogate(width=16) as net2, ppf.Simulation(shape, bc="periodic", precision="f32") as s2:
        net2.set_params(p)
        s2.upload(*st)
        net2.advance(s2, 1)
        ref = s2.download()
    for a, b in zip(got, ref):
        assert np.array_equal(a, b)
