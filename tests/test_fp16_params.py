"""Half-precision parameter storage (param_fp16): vp, epsilon and delta kept
as IEEE half in HBM, stencil and wavefields in FP32.

The kernels widen the halves and derive (vp dt)^2, 2 eps, 8 (eps - delta)
with the operations of the FP32 path, so a half-storage run equals an FP32
run on the half-rounded model bit for bit; the rounding itself is measured
against the FP64 oracle beside the FP32 run's error.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from helpers import bits_equal, rel_l2
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _rounded(shot):
    r = lambda a: a.astype(np.float16).astype(np.float32)
    return qp3d.Shot(shot.nx, shot.ny, shot.nz, shot.pml, shot.sz, shot.dx, shot.dy, shot.dz,
                     shot.dt, r(shot.vp), r(shot.eps), r(shot.delta), shot.src, shot.wavelet,
                     shot.prof, shot.c, shot.c2)


def _run(shot, fp16, **tune):
    with qp3d.Context(0) as ctx:
        ctx.tune(param_fp16=fp16, **tune)
        rec = ctx.forward(shot)
        ctx.load(shot)
        ctx.advance(shot.nt)
        return rec, ctx.record(), ctx.uxyzmax()


@pytest.mark.parametrize("threshold_mode", [1, 0])
def test_half_storage_equals_fp32_on_rounded_model(threshold_mode):
    shot = synthetic.small_case(hx=26, hy=22, nz0=20, pml=8, nt=70, seed=31)
    rec_h, rec_h2, mx_h = _run(shot, 1, threshold_mode=threshold_mode)
    rec_r, _, mx_r = _run(_rounded(shot), 0, threshold_mode=threshold_mode)
    assert bits_equal(rec_h, rec_r)
    assert bits_equal(rec_h2, rec_r)       # staged form too
    assert bits_equal(mx_h, mx_r)
    rec_f, _, _ = _run(shot, 0)
    assert not bits_equal(rec_h, rec_f)    # the rounding did happen


def test_half_storage_error_against_fp64():
    """The large workload's model decimated to the 200x200x100 copy its
    configuration names (every 4th cell: 40 m spacing), 10-cell PML, 5 Hz
    Ricker, 500 steps of 2 ms: the record of each parameter storage against
    FP64, beside the reference's own FP32 arithmetic (oracle REF32) on the
    same model, which the reference-arithmetic mode reproduces bit for bit.
    FP16 storage adds the rounding of the model itself (measured 1.45e-3,
    against 1.70e-5 for FP32 storage and 1.68e-5 for the reference's own
    FP32 arithmetic)."""
    shot = synthetic.large_vti(pml=10, nt=500, decimate=4, fm=5.0, dt=2e-3)
    rec_h, _, _ = _run(shot, 1)
    rec_f, _, _ = _run(shot, 0)
    rec_x, _, _ = _run(shot, 0, arith=0)
    prob = shot.to_oracle(O)
    r64, _, _ = O.run(O.F64, prob)
    r32, _, _ = O.run(O.REF32, prob)
    e_h, e_f, e_ref = rel_l2(rec_h, r64), rel_l2(rec_f, r64), rel_l2(r32, r64)
    print("large workload / 4 (200x200x100): record rel-L2 vs FP64: FP16 params %.3e, "
          "FP32 params %.3e (fast arithmetic), reference FP32 arithmetic %.3e; fast vs "
          "reference FP32 %.3e" % (e_h, e_f, e_ref, rel_l2(rec_f, r32)))
    assert bits_equal(rec_x, r32)
    assert e_f <= max(1e-5, 2 * e_ref)
    assert e_h <= 3e-3
    assert e_h > e_f
