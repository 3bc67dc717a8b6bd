"""Edge cases of the forward path against the oracle (GPU): no time steps, a
single step, the smallest grid the 10th-order stencil allows, no absorbing
layer, a layer thinner than the stencil's 5-cell band, extreme aspect
ratios, sources on the band and in corners.  Each record and max|grad u|
series must equal the oracle's mirror bit for bit, and qp3d_batch must give
the same records as one qp3d_forward per shot.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O
from helpers import bits_equal, rel_l2

pytestmark = pytest.mark.gpu

CASES = {
    # name: small_case arguments
    "one_step": dict(hx=22, hy=26, nz0=18, pml=8, nt=1, seed=21),
    "smallest_grid": dict(hx=11, hy=11, nz0=11, pml=0, nt=30, seed=22, src=(5, 5, 5)),
    "no_pml": dict(hx=22, hy=26, nz0=18, pml=0, nt=40, seed=23),
    "pml_3": dict(hx=20, hy=23, nz0=17, pml=3, nt=40, seed=24),
    "pml_5": dict(hx=20, hy=23, nz0=17, pml=5, nt=40, seed=25),
    "thin_x": dict(hx=1, hy=70, nz0=12, pml=6, nt=30, seed=26, src=(0, 35, 6)),
    "tall_z": dict(hx=12, hy=13, nz0=90, pml=6, nt=50, seed=27, src=(6, 6, 45)),
    "corner_source": dict(hx=21, hy=19, nz0=16, pml=7, nt=40, seed=28, src=(0, 0, 0)),
    "band_source": dict(hx=21, hy=19, nz0=16, pml=2, nt=40, seed=29, src=(10, 9, 0)),
    "ragged_y": dict(hx=17, hy=37, nz0=15, pml=6, nt=40, seed=30),
}


@pytest.fixture(scope="module")
def ctx():
    with qp3d.Context(0) as c:
        yield c


@pytest.mark.parametrize("name", sorted(CASES))
def test_edge_case_bit_exact_vs_mirror(ctx, name):
    shot = synthetic.small_case(**CASES[name])
    rec = ctx.forward(shot)
    ctx.load(shot)
    ctx.advance(shot.nt)
    mx = ctx.uxyzmax()
    prob = shot.to_oracle(O)
    mrec, mmx, _ = O.run(O.MIRROR, prob)
    assert rec.shape == (shot.nt, shot.hx, shot.hy)
    assert bits_equal(rec, mrec)
    assert bits_equal(mx, mmx)
    r32, _, _ = O.run(O.REF32, prob)
    if np.any(r32):
        assert rel_l2(rec, r32) <= 1e-5


def test_zero_steps(ctx):
    shot = synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=0, seed=31)
    rec = ctx.forward(shot)
    assert rec.shape == (0, shot.hx, shot.hy)
    ctx.load(shot)
    assert ctx.step == 0
    with pytest.raises(qp3d.QP3DError):
        ctx.advance(1)                 # past nt


def test_edge_cases_through_batch(ctx):
    names = ["one_step", "no_pml", "pml_5", "thin_x", "tall_z", "corner_source", "ragged_y",
             "no_steps"]
    shots = [synthetic.small_case(**CASES[n]) for n in names[:-1]]
    shots.append(synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=0, seed=31))
    single = [ctx.forward(s) for s in shots]
    recs = ctx.batch(shots)
    for n, a, b in zip(names, recs, single):
        assert bits_equal(a, b), n


def test_invalid_geometries_are_rejected(ctx):
    good = synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=5, seed=32)
    for field, value in (("nx", 10), ("ny", 10), ("nz", 10), ("pml", -1), ("sz", -1),
                         ("dx", 0.0), ("dt", -5e-4)):
        # the geometry check fires before any array is read
        bad = synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=5, seed=32)
        setattr(bad, field, value)
        with pytest.raises(qp3d.QP3DError):
            ctx.load(bad)
    bad = synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=5, seed=32)
    bad.sz = bad.nz
    with pytest.raises(qp3d.QP3DError):
        ctx.forward(bad)
    # the context still works
    rec = ctx.forward(good)
    assert rec.shape == (5, good.hx, good.hy)
