"""Failure paths on the GPU without a GPU fault: a bounded device-side wait
that runs out returns GPE_ERR_TIMEOUT, and the context stays usable.

The TMA-staged pass waits on mbarriers for its bulk copies with a bounded
poll.  GPE_TEST_TMA_STALL=<polls> (a test knob, read on every TMA launch)
makes each CTA arm its barriers for 16 bytes that are never issued and poll
only that many times: the wait runs out with no copy in flight, the CTA
raises the timeout and stop flags, and every later pass of the run returns
at once.  Nothing is left in flight when the CTAs exit, so the run ends
cleanly and the next call on the same context (knob unset) succeeds.
"""
import numpy as np
import pytest

from gpe_gb300._lib import GPE_ERR_TIMEOUT
from tests.test_gpu_parity import harmonic, rel_l2

pytestmark = pytest.mark.gpu


def make(gpe, variant):
    grid = gpe.grid3d(5, 32, 5, 32, 4, 32, precision="single")
    task = gpe.GPEtask(grid, harmonic((1.0, 1.2, 1.5)))
    task.set_pass_variant(variant)
    task.Ntotal, task.g, task.gamma = 20.0, 0.5, 0.01
    X, Y, Z = grid.mesh["x"], grid.mesh["y"], grid.mesh["z"]
    psi0 = (np.exp(-(X ** 2 + Y ** 2 + Z ** 2) / 2) * np.exp(0.2j * X)).astype(complex)
    return task, psi0


def test_tma_wait_timeout_returns_status_and_context_recovers(gpe, monkeypatch):
    task, psi0 = make(gpe, 1)  # TMA-staged passes
    monkeypatch.setenv("GPE_TEST_TMA_STALL", "64")
    task.init_state = psi0
    with pytest.raises(gpe.GPEError) as e:
        task.solve_split(0.002, 10, 1)
    assert e.value.status == GPE_ERR_TIMEOUT
    with pytest.raises(gpe.GPEError) as e:
        task.groundstate_itp(0.01, 1e-6, psi0)
    assert e.value.status == GPE_ERR_TIMEOUT

    # knob off: the same context and the same TMA passes run normally and
    # agree with a context on the direct passes
    monkeypatch.delenv("GPE_TEST_TMA_STALL")
    ref, _ = make(gpe, 0)
    for t in (task, ref):
        t.init_state = psi0
        t.current_iter = 0
        t.current_time = 0.0
        t.solve_split(0.002, 10, 2)
    assert rel_l2(task.current_state, ref.current_state) < 2e-5
    np.testing.assert_allclose(task.history["mu"], ref.history["mu"], rtol=2e-5)
    task.close()
    ref.close()
