"""qp3d_batch: many uneven shots in one time loop.

The batched launches share the tile bodies of the single-shot kernels, so
every record must equal qp3d_forward's for the same shot bit for bit (and
qp3d_forward is bit-identical to the mirror oracle, test_gpu_parity.py), in
every shape, graph, threshold and memory-group setting.
"""
import numpy as np
import pytest

import qp3d
import synthetic as S
from helpers import bits_equal

pytestmark = pytest.mark.gpu

# uneven grids, PML widths, receiver depths, source positions and nt
SPECS = [dict(hx=22, hy=26, nz0=18, pml=8, nt=60, seed=7),
         dict(hx=30, hy=17, nz0=24, pml=6, nt=52, seed=8),
         dict(hx=15, hy=40, nz0=12, pml=10, nt=60, seed=9, fm=25.0),
         dict(hx=41, hy=33, nz0=20, pml=5, nt=47, seed=10),
         dict(hx=20, hy=20, nz0=30, pml=7, nt=60, seed=11, src=(4, 15, 2))]


@pytest.fixture(scope="module")
def shots():
    return [S.small_case(**sp) for sp in SPECS]


@pytest.fixture(scope="module")
def expected(shots):
    with qp3d.Context(0) as ctx:
        return [ctx.forward(s) for s in shots]


def _same(recs, exp):
    assert len(recs) == len(exp)
    for i, (r, e) in enumerate(zip(recs, exp)):
        assert bits_equal(r, e), "shot %d differs from qp3d_forward" % i


def test_batch_matches_forward(shots, expected):
    with qp3d.Context(0) as ctx:
        recs = ctx.batch(shots)
        st = ctx.batch_stats()
        _same(recs, expected)
        assert st["batched_shots"] == len(shots) and st["single_shots"] == 0
        assert st["groups"] == 1
        assert st["tuned"] == 1 and st["ncand"] >= 2 and min(st["cand_ms"]) > 0
        assert st["graph_steps"] > 0
        # second call of the same sizes: cached shape, same records
        recs = ctx.batch(shots)
        st2 = ctx.batch_stats()
        _same(recs, expected)
        assert st2["tuned"] == 0 and st2["candidate"] == st["candidate"]


@pytest.mark.parametrize("setting", [
    dict(batch_tune=0, batch_candidate=0),
    dict(batch_tune=0, batch_candidate=2),
    dict(batch_tune=0, batch_candidate=3),
    dict(batch_tune=0, batch_candidate=4, batch_graph=0),
    dict(threshold_mode=0),
    dict(batch_mem_mb=1),
    dict(spec_bias_ppm=500000),
    dict(spec_delta_ppm=0),
])
def test_batch_settings(shots, expected, setting):
    with qp3d.Context(0) as ctx:
        ctx.tune(**setting)
        recs = ctx.batch(shots)
        st = ctx.batch_stats()
        _same(recs, expected)
        if setting.get("batch_mem_mb"):
            assert st["groups"] == len(shots)
        if setting.get("spec_bias_ppm"):
            assert st["redo_steps"] > 0
        if "batch_candidate" in setting:
            assert st["candidate"] == setting["batch_candidate"] and st["tuned"] == 0
        if setting.get("batch_graph", 1) == 0 or setting.get("threshold_mode", 1) == 0:
            assert st["graph_steps"] == 0


def test_batch_single_path_fallback(shots, expected):
    # a PML thinner than the 5-cell band puts the receivers outside the
    # updated box: that shot runs through qp3d_forward
    thin = S.small_case(hx=18, hy=18, nz0=16, pml=3, nt=40, seed=12)
    with qp3d.Context(0) as ctx:
        exp_thin = ctx.forward(thin)
        recs = ctx.batch(shots[:2] + [thin] + shots[2:3])
        st = ctx.batch_stats()
    _same(recs, expected[:2] + [exp_thin] + expected[2:3])
    assert st["single_shots"] == 1 and st["batched_shots"] == 3


def test_batch_errors(shots):
    with qp3d.Context(0) as ctx:
        bad = S.small_case(hx=18, hy=18, nz0=16, pml=4, nt=10, seed=13)
        bad.sz = bad.nz          # receiver plane outside the grid
        with pytest.raises(qp3d.QP3DError):
            ctx.batch([shots[0], bad])
        assert ctx.batch([]) == []
        # the context still works afterwards
        _ = ctx.batch(shots[:1])
