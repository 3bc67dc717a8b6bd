"""The reference's own GPU kernels (GPU_kernel.cu, compiled unmodified for
sm_103a) beside the CUDA path, the reference CPU arithmetic and FP64 (GPU).

The reference kernels are driven in the reference GPU driver's step sequence
(3dPureqPModeling_single_shot.cu:277-337) with zeroed buffers.  They compute
the same scheme as CPU_function.c but with nvcc's default contraction of a*b+c
into fused multiply-adds and double-precision literals in scalar_operator
(GPU_kernel.cu:87-115), so they are not bit-identical to the CPU operators;
every figure below is printed, and the bounds are the parity bounds of the
path (relative L2 <= 1e-5, max abs <= 1e-4 of the peak) where they hold for
the reference's own two implementations.
"""
import numpy as np
import pytest

import synthetic
from oracle import oracle as O
from helpers import FIXTURES, load_fixture, max_abs_rel_peak, plain_shot_oracles, rel_l2

pytestmark = [pytest.mark.gpu,
              pytest.mark.skipif(not O.ref_gpu_available(),
                                 reason="reference GPU kernels were not compiled")]


@pytest.mark.parametrize("name", FIXTURES)
def test_reference_gpu_golden(ctx, name):
    prob, shot, d = load_fixture(name)
    rec_ref, mx_ref, _, _ = O.run_reference_gpu(prob)
    rec_ref_h, mx_ref_h, _, _ = O.run_reference_gpu(prob, host_max=True)
    # the maximum does not depend on where it is taken
    assert np.array_equal(mx_ref, mx_ref_h) and np.array_equal(rec_ref, rec_ref_h)
    rec = ctx.forward(shot)
    r64, _, _ = O.run(O.F64, prob)
    e_cpu = rel_l2(rec_ref, d["record"])      # golden: the reference's CPU operators
    e_ours = rel_l2(rec, rec_ref)
    print("%s: GPU_kernel.cu vs CPU_function.c rel %.2e | CUDA path vs GPU_kernel.cu rel %.2e"
          " | vs FP64: GPU_kernel.cu %.2e, CUDA path %.2e, CPU_function.c %.2e" % (
              name, e_cpu, e_ours, rel_l2(rec_ref, r64), rel_l2(rec, r64),
              rel_l2(d["record"], r64)))
    assert e_cpu <= 1e-5 and max_abs_rel_peak(rec_ref, d["record"]) <= 1e-4
    assert e_ours <= 1e-5 and max_abs_rel_peak(rec, rec_ref) <= 1e-4


def test_reference_gpu_one_step_from_random_state(ctx):
    """Every PML face active: one step of the reference kernels against the
    CUDA path and the reference CPU arithmetic."""
    shot = synthetic.small_case(hx=24, hy=20, nz0=22, pml=9, nt=1, seed=4)
    u_prev, u_cur, pml_state = synthetic.random_state(shot, seed=4)
    prob = shot.to_oracle(O)

    def state():
        st = O.State(prob)
        st.u1[:] = u_prev
        st.u2[:] = u_cur
        st.u3[:] = u_cur
        st.pml[:] = pml_state
        return st

    _, _, sg, _ = O.run_reference_gpu(prob, state=state())
    _, _, s32 = O.run(O.REF32, prob, state=state())
    ctx.load(shot)
    ctx.write_state(0, u_prev, u_cur, pml_state)
    ctx.advance(1)
    _, g_cur, _ = ctx.read_state()
    e_cpu, e_ours = rel_l2(sg.u2, s32.u2), rel_l2(g_cur, sg.u2)
    print("one step: GPU_kernel.cu vs CPU_function.c rel %.2e, CUDA path vs GPU_kernel.cu %.2e"
          % (e_cpu, e_ours))
    assert e_cpu <= 1e-5 and e_ours <= 1e-5


def test_reference_gpu_plain_shot(ctx):
    """The reference CPU path's own workload (100^3 + 20-cell PML, 1000
    steps): the reference GPU kernels, the reference CPU arithmetic, FP64 and
    the CUDA path, every pair stated."""
    shot = synthetic.linear_vti()
    prob = shot.to_oracle(O)
    r32, r64 = plain_shot_oracles(shot)
    rg, _, _, ms = O.run_reference_gpu(prob)
    rec = ctx.forward(shot)
    pairs = {
        "GPU_kernel.cu vs CPU_function.c": (rg, r32),
        "GPU_kernel.cu vs FP64": (rg, r64),
        "CPU_function.c vs FP64": (r32, r64),
        "CUDA path vs GPU_kernel.cu": (rec, rg),
        "CUDA path vs CPU_function.c": (rec, r32),
        "CUDA path vs FP64": (rec, r64),
    }
    for k, (a, b) in pairs.items():
        print("plain shot: %-32s rel-L2 %.3e  max-abs/peak %.3e" % (k, rel_l2(a, b),
                                                                   max_abs_rel_peak(a, b)))
    print("plain shot: reference GPU kernels %.1f ms for 1000 steps (device max)" % ms)
    for a, b in pairs.values():
        assert max_abs_rel_peak(a, b) <= 1e-4
