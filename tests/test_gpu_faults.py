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
