"""Failure paths on the GPU without a fault: a bounded device wait that runs
out reports NN_ERR_TIMEOUT and leaves the context usable; a request over the
context's HBM budget is refused with NN_ERR_BUDGET before anything runs."""
import numpy as np
import pytest

from natural_number_gb300.synth import limbs

pytestmark = pytest.mark.gpu


def test_lookback_wait_times_out_and_context_recovers(oracle):
    import natural_number_gb300 as nn
    ctx = nn.Context(0)
    a, b = limbs(41, 3000), limbs(42, 2500)
    assert np.array_equal(ctx.mul(a, b), oracle.mul(a, b))
    # a status word nothing sets: the wait gives up after 1000 polls
    assert ctx.probe_wait(1000) == nn.NN_ERR_TIMEOUT
    assert "wait" in nn.lib().nn_last_error(ctx.h).decode()
    # the error was reported once and cleared; the context still multiplies
    ctx.synchronize()
    assert np.array_equal(ctx.mul(b, a), oracle.mul(b, a))
    assert ctx.probe_wait(1) == nn.NN_ERR_TIMEOUT
    ctx.synchronize()
    ctx.close()


def test_budget_refuses_oversize_product(oracle):
    import natural_number_gb300 as nn
    # staging for the operands and product takes 32 MiB; the two 48 MiB
    # transforms of a 2^20 x 2^20 product would go over a 48 MiB budget
    ctx = nn.Context(0, hbm_budget=48 << 20)
    a, b = limbs(5, 1 << 20), limbs(6, 1 << 20)
    with pytest.raises(nn.NNError) as e:
        ctx.mul(a, b)
    assert e.value.status == nn.NN_ERR_BUDGET
    small_a, small_b = limbs(7, 5000), limbs(8, 4000)
    assert np.array_equal(ctx.mul(small_a, small_b), oracle.mul(small_a, small_b))
    ctx.close()
