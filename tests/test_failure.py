"""Bounded device waits (GPU): a wait that runs out is reported, and the
context keeps working.

Every wait of the kernels on an mbarrier (a staged plane, a released slot)
gives up after a limit ("wait_limit_us", default 2 s), sets an error bit,
waits (bounded) for its own copies in flight and returns; the host reports
QP3D_ERR_TIMEOUT.  A test hook ("test_hold_plane") keeps one plane of the
first CTA from ever being loaded, so that its waits run out: nothing faults
or hangs, and with the hook cleared the same context computes the shot
exactly as before.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from helpers import bits_equal

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mode", [0, 1])
def test_wait_that_runs_out_is_reported_and_recovered(ctx, mode):
    shot = synthetic.small_case(hx=26, hy=22, nz0=20, pml=7, nt=12, seed=17)
    ctx.tune(threshold_mode=mode)
    want = ctx.forward(shot)
    try:
        ctx.tune(wait_limit_us=20000, test_hold_plane=2)
        assert ctx.tuning("wait_limit_us") == 20000 and ctx.tuning("test_hold_plane") == 2
        ctx.load(shot)
        ctx.advance(4)          # gradmax pre-pass steps, then speculative ones
        with pytest.raises(qp3d.QP3DError, match="-4"):
            ctx.sync()
    finally:
        ctx.tune(wait_limit_us=0, test_hold_plane=-1, threshold_mode=1)
    ctx.reset()
    ctx.advance(shot.nt)
    assert bits_equal(ctx.record(), want)
