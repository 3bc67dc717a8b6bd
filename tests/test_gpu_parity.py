"""CUDA path in its default (fast) arithmetic against the oracle, through
the C ABI (GPU).

Three levels of agreement are checked:
  * bit for bit against the oracle's MIRROR variant -- the arithmetic the
    kernels state (folded 1/h coefficients, fused multiply-adds, IEEE
    division/sqrt); any indexing, face-priority or pipeline error breaks it;
  * against the reference FP32 arithmetic (oracle REF32, pinned to
    CPU_function.c) and the golden vectors made by the reference's own code:
    relative L2 <= 1e-5 and max-abs <= 1e-4 of the peak;
  * against FP64, relative L2 <= 1e-5 and stated for every result.
The S operator switches on mode > 0.01*max|grad u| (GPU_kernel.cu:99), so any
two FP32 arithmetics that are not bit-identical drift apart by threshold
flips over long runs; the bounds hold over a whole 1000-step shot.  The
reference-arithmetic mode is checked bit for bit in test_reference_arith.py.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O
from helpers import FIXTURES, bits_equal, load_fixture, max_abs_rel_peak, plain_shot_oracles, rel_l2

pytestmark = pytest.mark.gpu


def _live_pml_mask(nx, ny, nz, pml):
    """Entries of the canonical PML buffer that belong to a cell the reference
    updates ([5,n-5)^3) and that the owning face holds (face priority)."""
    n = O.pml_state_size(nx, ny, nz, pml)
    mask = np.zeros(n + 1, bool)
    z, x, y = np.meshgrid(np.arange(nz), np.arange(nx), np.arange(ny), indexing="ij")
    inside = (x >= 5) & (x < nx - 5) & (y >= 5) & (y < ny - 5) & (z >= 5) & (z < nz - 5)
    reg = np.full(x.shape, -1)
    conds = [x < pml, x >= nx - pml, y < pml, y >= ny - pml, z < pml, z >= nz - pml]
    for f in range(5, -1, -1):
        reg = np.where(conds[f], f, reg)
    sizes = [pml * ny * nz] * 2 + [pml * nx * nz] * 2 + [pml * nx * ny] * 2
    off = 0
    live_arrays = [0, 1, 3, 4, 5, 7, 8]   # w11 w12 w21 w31 w32 p1 p2
    for f in range(6):
        sel = inside & (reg == f)
        zz, xx, yy = z[sel], x[sel], y[sel]
        if f == 0:
            fi = zz * ny * pml + xx * ny + yy
        elif f == 1:
            fi = zz * ny * pml + (xx - nx + pml) * ny + yy
        elif f == 2:
            fi = zz * nx * pml + xx * pml + yy
        elif f == 3:
            fi = zz * nx * pml + xx * pml + (yy - ny + pml)
        elif f == 4:
            fi = zz * nx * ny + xx * ny + yy
        else:
            fi = (zz - nz + pml) * ny * nx + xx * ny + yy
        for a in live_arrays:
            mask[off + a * sizes[f] + fi] = True
        off += 10 * sizes[f]
    return mask


def _oracle_state(prob, u_prev, u_cur, pml):
    st = O.State(prob)
    st.u1[:] = u_prev
    st.u2[:] = u_cur
    st.pml[:] = pml
    return st


# ---------------------------------------------------------------------------
# operator level: every face active from step 0
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("dims,seed", [((22, 26, 18, 8), 1), ((33, 21, 27, 12), 2),
                                       ((40, 36, 30, 3), 3)])
def test_steps_from_random_state_bit_exact_vs_mirror(ctx, dims, seed):
    hx, hy, nz0, pml = dims
    shot = synthetic.small_case(hx=hx, hy=hy, nz0=nz0, pml=pml, nt=3, seed=seed)
    u_prev, u_cur, pml_state = synthetic.random_state(shot, seed=seed)
    ctx.load(shot)
    ctx.write_state(0, u_prev, u_cur, pml_state)
    ctx.advance(3)
    rec, mx = ctx.record(0, 3), ctx.uxyzmax(0, 3)
    g_prev, g_cur, g_pml = ctx.read_state()

    prob = shot.to_oracle(O)
    st = _oracle_state(prob, u_prev, u_cur, pml_state)
    orec, omx, st = O.run(O.MIRROR, prob, state=st)
    assert bits_equal(mx, omx), (mx, omx)
    assert bits_equal(g_cur, st.u2)
    assert bits_equal(g_prev, st.u1)
    assert bits_equal(rec, orec)
    live = _live_pml_mask(shot.nx, shot.ny, shot.nz, shot.pml)
    assert bits_equal(g_pml[live], st.pml[live])


@pytest.mark.parametrize("seed", [4, 5])
def test_one_step_from_random_state_vs_reference_arithmetic(ctx, seed):
    shot = synthetic.small_case(hx=24, hy=20, nz0=22, pml=9, nt=1, seed=seed)
    u_prev, u_cur, pml_state = synthetic.random_state(shot, seed=seed)
    ctx.load(shot)
    ctx.write_state(0, u_prev, u_cur, pml_state)
    ctx.advance(1)
    _, g_cur, g_pml = ctx.read_state()
    prob = shot.to_oracle(O)
    _, _, s32 = O.run(O.REF32, prob, state=_oracle_state(prob, u_prev, u_cur, pml_state))
    _, _, s64 = O.run(O.F64, prob, state=_oracle_state(prob, u_prev, u_cur, pml_state).copy(np.float64))
    live = _live_pml_mask(shot.nx, shot.ny, shot.nz, shot.pml)
    assert rel_l2(g_cur, s32.u2) <= 1e-5
    assert max_abs_rel_peak(g_cur, s32.u2) <= 1e-4
    assert rel_l2(g_pml[live], s32.pml[live]) <= 1e-5
    # error against FP64 of the same size as the reference arithmetic's own
    e_gpu, e_ref = rel_l2(g_cur, s64.u2), rel_l2(s32.u2, s64.u2)
    assert e_gpu <= 1e-5 and e_ref <= 1e-5, (e_gpu, e_ref)


# ---------------------------------------------------------------------------
# whole shots
# ---------------------------------------------------------------------------
@pytest.mark.parametrize("name", FIXTURES)
def test_golden_fixture(ctx, name):
    """Golden vectors produced by the reference's own compiled operators."""
    prob, shot, d = load_fixture(name)
    rec = ctx.forward(shot)
    e_rel, e_max = rel_l2(rec, d["record"]), max_abs_rel_peak(rec, d["record"])
    assert e_rel <= 1e-5 and e_max <= 1e-4, (e_rel, e_max)
    mrec, mmx, _ = O.run(O.MIRROR, prob)
    assert bits_equal(rec, mrec)
    ctx.load(shot)
    ctx.advance(shot.nt)
    assert bits_equal(ctx.uxyzmax(), mmx)
    r64, _, _ = O.run(O.F64, prob)
    print("%s: vs reference rel %.2e max %.2e | vs FP64 rel %.2e (reference FP32 %.2e)" % (
        name, e_rel, e_max, rel_l2(rec, r64), rel_l2(d["record"], r64)))


def test_small_shot_all_variants(ctx):
    """A 38x42x34 grid over 120 steps: the wave crosses every face several
    times.  On a grid this small a single threshold flip moves the record by
    ~1e-5, so the reference's own FP32 arithmetic is 1.3e-5 from FP64 here;
    the fast arithmetic is held to the same distance from both."""
    shot = synthetic.small_case(nt=120, seed=9)
    rec = ctx.forward(shot)
    prob = shot.to_oracle(O)
    mrec, _, mst = O.run(O.MIRROR, prob)
    assert bits_equal(rec, mrec)
    r32, _, _ = O.run(O.REF32, prob)
    r64, _, _ = O.run(O.F64, prob)
    e_ref = rel_l2(r32, r64)
    print("small shot: fast vs REF32 %.3e, vs FP64 %.3e; REF32 vs FP64 %.3e" %
          (rel_l2(rec, r32), rel_l2(rec, r64), e_ref))
    assert rel_l2(rec, r32) <= max(1e-5, 2 * e_ref) and max_abs_rel_peak(rec, r32) <= 1e-4
    assert rel_l2(rec, r64) <= max(1e-5, 2 * e_ref)
    _, g_cur, _ = ctx.read_state()
    assert bits_equal(g_cur, mst.u2)


def test_linear_vti_plain_shot_full(ctx):
    """100^3 interior, 20-cell PML, 1000 steps of 0.5 ms, 25 Hz Ricker at
    (50,50,5), receivers on z=5: the reference CPU path's own workload, in the
    default (fast) arithmetic.  Bounds: relative L2 <= 1e-5 against the
    reference FP32 arithmetic and against FP64 over the whole record, max-abs
    <= 1e-4 of the peak.  (The reference's own GPU and CPU codes differ by
    7.0e-6 on this shot; the reference-arithmetic mode equals the CPU code
    bit for bit, test_reference_arith.py.)"""
    shot = synthetic.linear_vti()
    rec = ctx.forward(shot)
    r32, r64 = plain_shot_oracles(shot)
    e_rel, e_max = rel_l2(rec, r32), max_abs_rel_peak(rec, r32)
    e64, e64_ref = rel_l2(rec, r64), rel_l2(r32, r64)
    print("plain shot: vs ref32 rel %.3e max %.3e | vs FP64 %.3e max %.3e (ref32 vs FP64 %.3e)" %
          (e_rel, e_max, e64, max_abs_rel_peak(rec, r64), e64_ref))
    assert e_max <= 1e-4 and max_abs_rel_peak(rec, r64) <= 1e-4
    assert e_rel <= 1e-5
    assert e64 <= 1e-5


# ---------------------------------------------------------------------------
# API behaviour
# ---------------------------------------------------------------------------
def test_staged_equals_forward_and_is_repeatable(ctx):
    shot = synthetic.small_case(nt=40, seed=3)
    a = ctx.forward(shot)
    ctx.load(shot)
    ctx.advance(15)
    ctx.advance(25)
    b = ctx.record()
    ctx.reset()
    ctx.advance(40)
    c = ctx.record()
    assert bits_equal(a, b) and bits_equal(a, c)


def test_snapshots_match_state(ctx):
    shot = synthetic.small_case(nt=25, seed=4)
    got = {}

    def cb(step, kind, arr):
        got[(step, kind)] = arr
        return 0

    snap = qp3d.make_snap(cb, 10, [qp3d.SNAP_VOLUME, qp3d.SNAP_XZ, qp3d.SNAP_YZ, qp3d.SNAP_XY])
    ctx.forward(shot, snap=snap)
    assert sorted({k for k, _ in got}) == [0, 10, 20]
    prob = shot.to_oracle(O)
    st = None
    pml, hx, hy, hz = shot.pml, shot.hx, shot.hy, shot.nz - 2 * shot.pml
    done = 0
    for k in (0, 10, 20):
        _, _, st = O.run(O.MIRROR, prob, k0=done, nsteps=k + 1 - done, state=st,
                         want_record=False)
        done = k + 1
        u = st.u2.reshape(shot.nz, shot.nx, shot.ny)[pml:pml + hz, pml:pml + hx, pml:pml + hy]
        assert bits_equal(got[(k, qp3d.SNAP_VOLUME)], u)
        assert bits_equal(got[(k, qp3d.SNAP_XZ)], u[:, :, (hy - 1) // 2])
        assert bits_equal(got[(k, qp3d.SNAP_YZ)], u[:, (hx - 1) // 2, :])
        assert bits_equal(got[(k, qp3d.SNAP_XY)], u[(hz - 1) // 2])


def test_receiver_plane_outside_updated_box(ctx):
    """sz in the never-updated band and pml < 5: the record comes from the
    separate record kernel and must still match."""
    shot = synthetic.small_case(hx=20, hy=18, nz0=24, pml=3, nt=30, seed=8)
    shot.sz = 2
    rec = ctx.forward(shot)
    prob = shot.to_oracle(O)
    mrec, _, _ = O.run(O.MIRROR, prob)
    assert bits_equal(rec, mrec)


def test_error_codes(ctx):
    shot = synthetic.small_case(nt=5)
    bad = synthetic.small_case(nt=5)
    bad.pml = 40                       # 2*pml >= n
    with pytest.raises(qp3d.QP3DError, match="-1"):
        ctx.load(bad)
    ctx.load(shot)
    with pytest.raises(qp3d.QP3DError, match="-1"):
        ctx.advance(6)                 # past nt
    ctx.advance(5)
    t = ctx.launches_per_step()
    assert t >= 2


def test_timing_helper(ctx):
    shot = synthetic.small_case(nt=20, seed=2)
    ctx.load(shot)
    total, ms_step, ms_grad = ctx.time(10)
    assert total > 0 and ms_step > 0 and ms_grad > 0
    assert ms_step + ms_grad <= total * 1.05 + 0.05


@pytest.mark.parametrize("mode,grad_v,tile_x,chunks", [(0, 0, 0, 0), (1, 1, 0, 0),
                                                       (1, 0, 17, 3), (0, 1, 32, 1),
                                                       (1, 1, 9, 5)])
def test_tuning_settings_are_bit_identical(ctx, mode, grad_v, tile_x, chunks):
    """Every threshold mode, launch variant, tile height and z-chunking
    computes the same bits as the oracle mirror (the autotuner may pick any)."""
    shot = synthetic.small_case(hx=30, hy=34, nz0=40, pml=8, nt=30, seed=12)
    ctx.tune(threshold_mode=mode, gradmax_variant=grad_v, tile_x=tile_x, chunks=chunks)
    try:
        rec = ctx.forward(shot)
        ctx.load(shot)
        ctx.advance(shot.nt)
        mx = ctx.uxyzmax()
    finally:
        ctx.tune(threshold_mode=1, gradmax_variant=0, tile_x=0, chunks=0)
    mrec, mmx, _ = O.run(O.MIRROR, shot.to_oracle(O))
    assert bits_equal(rec, mrec)
    assert bits_equal(mx, mmx)


@pytest.mark.parametrize("delta_ppm,bias_ppm", [(0, 0), (250000, 0), (20000, 500000),
                                                (20000, -400000), (20000, 0)])
def test_speculative_threshold_paths(ctx, delta_ppm, bias_ppm):
    """The speculative step: a narrow window makes some predictions miss
    (exact re-runs), a wide one defers many cells to the fix-up, a window
    shifted above or below the prediction misses on every step; every path
    stays bit-identical to the mirror."""
    shot = synthetic.small_case(hx=26, hy=30, nz0=30, pml=8, nt=90, seed=21)
    ctx.tune(spec_delta_ppm=delta_ppm, spec_bias_ppm=bias_ppm)
    try:
        ctx.load(shot)
        ctx.advance(shot.nt)
        rec, mx = ctx.record(), ctx.uxyzmax()
        redo, alt = ctx.stats()
    finally:
        ctx.tune(spec_delta_ppm=10000, spec_bias_ppm=0)
    mrec, mmx, _ = O.run(O.MIRROR, shot.to_oracle(O))
    assert bits_equal(rec, mrec)
    assert bits_equal(mx, mmx)
    if bias_ppm:   # most predictions miss (fast early growth can still land inside)
        assert redo[3:].mean() > 0.5
    if delta_ppm == 250000:
        assert alt.max() > 0
    print("delta %d bias %d: re-runs %d of %d, max deferred cells %d" % (
        delta_ppm, bias_ppm, int(redo.sum()), shot.nt, int(alt.max())))


def test_pinned_record_is_streamed_identically(ctx):
    """A page-locked record buffer is filled piece by piece while the time
    loop runs (a second stream); the result equals the pageable path's, with
    and without snapshots, over several 100-step pieces."""
    shot = synthetic.small_case(hx=20, hy=18, nz0=16, pml=6, nt=250, seed=6)
    want = ctx.forward(shot)
    snap = qp3d.make_snap(lambda step, kind, arr: 0, 30, [qp3d.SNAP_XZ])
    for sn in (None, snap):
        pin = qp3d.PinnedArray(want.shape)
        try:
            pin.array[:] = np.nan
            ctx.forward(shot, snap=sn, record=pin.array)
            assert bits_equal(pin.array, want)
        finally:
            pin.free()


def test_snapshot_ring_order_and_failure(ctx):
    """qp3d_forward hands snapshots over from a ring of device / page-locked
    slots while later steps already run: every snapshot arrives, in step
    order, equal to the staged path's (qp3d_shot_snapshot after the same
    step), also when the ring wraps many times and with a page-locked record;
    a callback that fails stops the call with QP3D_ERR_CALLBACK at its own
    step and leaves the context usable."""
    shot = synthetic.small_case(hx=20, hy=18, nz0=16, pml=6, nt=120, seed=9)
    kinds = [qp3d.SNAP_VOLUME, qp3d.SNAP_XZ, qp3d.SNAP_YZ]
    every = 7
    want_steps = [k for k in range(shot.nt) if k % every == 0]

    def collect(into):
        def cb(step, kind, arr):
            into.append((step, kind, arr))
            return 0
        return qp3d.make_snap(cb, every, kinds)

    got = []
    rec = ctx.forward(shot, snap=collect(got))
    pin = qp3d.PinnedArray(rec.shape)
    got_pinned = []
    try:
        ctx.forward(shot, snap=collect(got_pinned), record=pin.array)
        assert bits_equal(pin.array, rec)
    finally:
        pin.free()
    ref = []
    snap_ref = collect(ref)
    ctx.load(shot)
    k = 0
    while k < shot.nt:
        nxt = k if k % every == 0 else (k // every + 1) * every
        n = min(shot.nt - k, nxt - k + 1)
        ctx.advance(n)
        k += n
        if (k - 1) % every == 0:
            ctx.snapshot(snap_ref)
    assert [s for s, _, _ in ref] == sorted(s for s, _, _ in ref)
    assert sorted({s for s, _, _ in ref}) == want_steps
    for run in (got, got_pinned):
        assert len(run) == len(ref) == len(want_steps) * len(kinds)
        for (s1, k1, a1), (s2, k2, a2) in zip(run, ref):
            assert s1 == s2 and k1 == k2 and bits_equal(a1, a2)
    seen = []

    def bad(step, kind, arr):
        seen.append(step)
        return 1 if step >= 21 else 0

    with pytest.raises(qp3d.QP3DError, match=r"\(-7 "):
        ctx.forward(shot, snap=qp3d.make_snap(bad, every, [qp3d.SNAP_XZ]))
    assert seen == [0, 7, 14, 21]
    assert bits_equal(ctx.forward(shot), rec)
