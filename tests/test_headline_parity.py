"""Parity on the headline workload (GPU): the 400x400x300 layered model with
a 30-cell PML (460x460x360 padded cells, 12 dipping layers, vp 1500-4500 m/s,
eps up to 0.3, 20 Hz Ricker at the surface centre), the first 300 of its 3000
steps.  The full 400x400 surface record and the xz / yz mid slices at steps
0, 100 and 200 are compared:
  * reference-arithmetic mode: bit for bit against the reference CPU
    operators (oracle REF32, pinned to CPU_function.c);
  * default fast arithmetic: relative L2 <= 1e-5 and max-abs <= 1e-4 of the
    peak against REF32 and against FP64.
The CPU oracles take a few minutes on the host cores.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O
from helpers import bits_equal, max_abs_rel_peak, rel_l2

pytestmark = pytest.mark.gpu

NT = 300
SNAPS = (0, 100, 200)


def _gpu(shot, arith):
    got = {}

    def cb(step, kind, arr):
        got[(step, kind)] = np.array(arr, copy=True)
        return 0

    snap = qp3d.make_snap(cb, 100, [qp3d.SNAP_XZ, qp3d.SNAP_YZ])
    with qp3d.Context(0) as ctx:
        ctx.tune(arith=arith)
        rec = ctx.forward(shot, snap=snap)
    return rec, got


def _oracle(shot, variant):
    prob = shot.to_oracle(O)
    dt = np.float64 if variant == O.F64 else np.float32
    st = O.State(prob, dt)
    recs, slices, done = [], {}, 0
    hx, hy, pml = shot.hx, shot.hy, shot.pml
    hz = shot.nz - 2 * pml
    for k in SNAPS + (NT - 1,):
        r, _, st = O.run(variant, prob, k0=done, nsteps=k + 1 - done, state=st)
        recs.append(r)
        done = k + 1
        if k in SNAPS:
            u = st.u2.reshape(shot.nz, shot.nx, shot.ny)[pml:pml + hz, pml:pml + hx, pml:pml + hy]
            slices[(k, qp3d.SNAP_XZ)] = u[:, :, (hy - 1) // 2].copy()
            slices[(k, qp3d.SNAP_YZ)] = u[:, (hx - 1) // 2, :].copy()
    return np.concatenate(recs), slices


@pytest.fixture(scope="module")
def headline():
    shot = synthetic.layered_vti(nt=NT)
    r32, s32 = _oracle(shot, O.REF32)
    r64, s64 = _oracle(shot, O.F64)
    return shot, r32, s32, r64, s64


def test_headline_reference_arithmetic_bit_exact(headline):
    shot, r32, s32, _, _ = headline
    rec, sl = _gpu(shot, 0)
    ndiff = int(np.count_nonzero(rec.view(np.uint32) != r32.view(np.uint32)))
    print("headline, reference arithmetic: %d of %d record samples differ" % (ndiff, rec.size))
    assert ndiff == 0
    for key, want in s32.items():
        assert bits_equal(sl[key], want), key


def test_headline_fast_arithmetic_bounds(headline):
    shot, r32, s32, r64, s64 = headline
    rec, sl = _gpu(shot, 1)
    e32, e64 = rel_l2(rec, r32), rel_l2(rec, r64)
    m32, m64 = max_abs_rel_peak(rec, r32), max_abs_rel_peak(rec, r64)
    print("headline record: fast vs REF32 rel %.3e max %.3e | vs FP64 rel %.3e max %.3e | "
          "REF32 vs FP64 rel %.3e" % (e32, m32, e64, m64, rel_l2(r32, r64)))
    assert e32 <= 1e-5 and e64 <= 1e-5 and m32 <= 1e-4 and m64 <= 1e-4
    for key in s32:
        a32, a64 = rel_l2(sl[key], s32[key]), rel_l2(sl[key], s64[key])
        print("headline slice step %d kind %d: vs REF32 %.3e, vs FP64 %.3e" % (key[0], key[1],
                                                                             a32, a64))
        assert a32 <= 1e-5 and a64 <= 1e-5
        assert max_abs_rel_peak(sl[key], s32[key]) <= 1e-4
