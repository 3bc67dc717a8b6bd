"""The kernels in their reference-arithmetic mode ("arith" = 0) against the
reference CPU operators, bit for bit (GPU).

In this mode every float operation of CPU_function.c:301-480 is the same
IEEE operation in the same order (each stencil tap divided by dx or dx*dx,
the taps summed from zero, the double-precision parts of the scalar operator
and of the PML update reproduced exactly), so the CUDA path must equal the
oracle's REF32 variant -- pinned bit for bit to the reference's own compiled
CPU_function.c -- in every record sample, every per-step maximum and every
state value, through the speculative threshold, the fused sources and the
batched launches.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O
from helpers import FIXTURES, bits_equal, load_fixture, plain_shot_oracles

pytestmark = pytest.mark.gpu

REF = 0   # "arith" tuning value of the reference arithmetic


@pytest.fixture
def rctx(ctx):
    ctx.tune(arith=REF)
    yield ctx
    ctx.tune(arith=1, threshold_mode=1, spec_delta_ppm=10000, spec_bias_ppm=0, param_fp16=0)


def _live_pml(shot):
    from test_gpu_parity import _live_pml_mask
    return _live_pml_mask(shot.nx, shot.ny, shot.nz, shot.pml)


@pytest.mark.parametrize("name", FIXTURES)
def test_golden_fixture_bit_exact(rctx, name):
    """Golden vectors made by the reference's own compiled operators."""
    prob, shot, d = load_fixture(name)
    rec = rctx.forward(shot)
    assert bits_equal(rec, d["record"])
    rctx.load(shot)
    rctx.advance(shot.nt)
    assert bits_equal(rctx.uxyzmax(), d["uxyzmax"])
    g_prev, g_cur, g_pml = rctx.read_state()
    assert bits_equal(g_cur, d["u_cur"]) and bits_equal(g_prev, d["u_prev"])
    live = _live_pml(shot)
    assert bits_equal(g_pml[live], d["pml_state"][live])


@pytest.mark.parametrize("dims,seed", [((22, 26, 18, 8), 1), ((33, 21, 27, 12), 2),
                                       ((40, 36, 30, 3), 3)])
def test_random_states_bit_exact(rctx, dims, seed):
    """Every PML face active and gradients on both sides of the threshold."""
    hx, hy, nz0, pml = dims
    shot = synthetic.small_case(hx=hx, hy=hy, nz0=nz0, pml=pml, nt=4, seed=seed)
    u_prev, u_cur, pml_state = synthetic.random_state(shot, seed=seed)
    rctx.load(shot)
    rctx.write_state(0, u_prev, u_cur, pml_state)
    rctx.advance(4)
    rec, mx = rctx.record(0, 4), rctx.uxyzmax(0, 4)
    g_prev, g_cur, g_pml = rctx.read_state()
    prob = shot.to_oracle(O)
    st = O.State(prob)
    st.u1[:], st.u2[:], st.u3[:], st.pml[:] = u_prev, u_cur, u_cur, pml_state
    orec, omx, st = O.run(O.REF32, prob, state=st)
    assert bits_equal(mx, omx)
    assert bits_equal(rec, orec)
    assert bits_equal(g_cur, st.u2) and bits_equal(g_prev, st.u1)
    live = _live_pml(shot)
    assert bits_equal(g_pml[live], st.pml[live])


def test_plain_shot_bit_exact(rctx):
    """The reference CPU path's own workload (100^3 + 20-cell PML, 1000 steps
    of 0.5 ms, 25 Hz Ricker): every record sample equal to CPU_function.c's."""
    shot = synthetic.linear_vti()
    rec = rctx.forward(shot)
    r32, _ = plain_shot_oracles(shot)
    ndiff = int(np.count_nonzero(rec.view(np.uint32) != r32.view(np.uint32)))
    print("plain shot, reference arithmetic: %d of %d record samples differ" % (ndiff, rec.size))
    assert ndiff == 0


@pytest.mark.parametrize("mode,delta_ppm,bias_ppm", [(0, 10000, 0), (1, 250000, 0),
                                                     (1, 20000, 500000), (1, 20000, -400000)])
def test_threshold_paths_bit_exact(rctx, mode, delta_ppm, bias_ppm):
    """Gradmax pre-pass, wide windows (many deferred cells fixed up) and
    windows that miss on every step (exact re-runs) all give the reference's
    bits."""
    shot = synthetic.small_case(hx=26, hy=30, nz0=30, pml=8, nt=90, seed=21)
    rctx.tune(threshold_mode=mode, spec_delta_ppm=delta_ppm, spec_bias_ppm=bias_ppm)
    rctx.load(shot)
    rctx.advance(shot.nt)
    rec, mx = rctx.record(), rctx.uxyzmax()
    r32, m32, _ = O.run(O.REF32, shot.to_oracle(O))
    assert bits_equal(mx, m32)
    assert bits_equal(rec, r32)


def test_batch_bit_exact(rctx):
    """qp3d_batch in the reference arithmetic: uneven shots, each equal to
    the reference CPU operators' record."""
    shots = [synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=60, seed=7),
             synthetic.small_case(hx=18, hy=24, nz0=16, pml=6, nt=50, seed=2),
             synthetic.small_case(hx=30, hy=20, nz0=22, pml=9, nt=40, seed=5)]
    recs = rctx.batch(shots)
    for s, r in zip(shots, recs):
        r32, _, _ = O.run(O.REF32, s.to_oracle(O))
        assert bits_equal(r, r32)


def test_fp16_parameters_bit_exact(rctx):
    """Half-precision parameter storage in the reference arithmetic equals the
    reference CPU operators on the half-rounded model."""
    shot = synthetic.small_case(hx=24, hy=22, nz0=20, pml=7, nt=50, seed=13)
    rctx.tune(param_fp16=1)
    rec = rctx.forward(shot)
    rctx.tune(param_fp16=0)
    h = lambda a: np.asarray(a, np.float32).astype(np.float16).astype(np.float32)
    half = qp3d.Shot(shot.nx, shot.ny, shot.nz, shot.pml, shot.sz, shot.dx, shot.dy, shot.dz,
                     shot.dt, h(shot.vp), h(shot.eps), h(shot.delta), shot.src, shot.wavelet,
                     shot.prof, shot.c, shot.c2)
    r32, _, _ = O.run(O.REF32, half.to_oracle(O))
    assert bits_equal(rec, r32)
