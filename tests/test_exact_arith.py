"""The library's exact-arithmetic header (csrc/qp3d_exact.h), compiled for the
CPU, against the oracle's restatement of the reference CPU operators (REF32,
pinned bit for bit to CPU_function.c): whole runs equal bit for bit, the
scalar operator equals the reference's double expression on millions of
random gradients, and the FP64 fallbacks stay rare.  The header's
approximations (reciprocal, reciprocal square root) are also run perturbed
by 2^-21 relative, more than the device instructions' error, to show that
the results do not depend on them.
"""
import ctypes
import os
import subprocess

import numpy as np
import pytest

import synthetic
from oracle import oracle as O
from helpers import FIXTURES, bits_equal, load_fixture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "gpu-c_3dqmodeling_gb300", "csrc")


def _build(tmp, skew):
    src = os.path.join(os.path.dirname(os.path.abspath(__file__)), "exact_emul.cpp")
    out = os.path.join(str(tmp), "libemul_%s.so" % ("skew" if skew else "plain"))
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp",
           "-I", CSRC, "-I", os.path.join(ROOT, "oracle"), "-o", out, src, "-lm"]
    if skew:
        cmd.insert(1, "-DQP3D_XR_APPROX_SKEW=%r" % skew)
    subprocess.check_call(cmd)
    L = ctypes.CDLL(out)
    L.emul_run.restype = ctypes.c_int
    L.emul_run.argtypes = ([ctypes.POINTER(O.OracleArgs), ctypes.c_int, ctypes.c_int] +
                           [ctypes.c_void_p] * 7)
    L.emul_check_scalar.restype = ctypes.c_longlong
    L.emul_check_scalar.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_longlong] + \
        [ctypes.c_void_p] * 2
    L.emul_fallback_rates.argtypes = [ctypes.c_void_p] * 5 + [ctypes.c_longlong] + \
        [ctypes.c_void_p] * 2
    return L


@pytest.fixture(scope="module", params=[0.0, 2.0 ** -21], ids=["exact-approx", "skewed-approx"])
def emul(request, tmp_path_factory):
    return _build(tmp_path_factory.mktemp("emul"), request.param)


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def emul_run(L, prob, state=None, k0=0, nsteps=None):
    if nsteps is None:
        nsteps = prob.nt - k0
    if state is None:
        state = O.State(prob)
    hx, hy = prob.nx - 2 * prob.pml, prob.ny - 2 * prob.pml
    rec = np.zeros((nsteps, hx, hy), np.float32)
    mx = np.zeros(nsteps, np.float32)
    cnt = np.zeros(2, np.int64)
    args = prob.args()
    rc = L.emul_run(ctypes.byref(args), k0, nsteps, _p(state.u1), _p(state.u2), _p(state.u3),
                    _p(state.pml), _p(rec), _p(mx), _p(cnt))
    assert rc == 0
    return rec, mx, state, cnt


def _same_state(a, b):
    return (bits_equal(a.u1, b.u1) and bits_equal(a.u2, b.u2) and bits_equal(a.u3, b.u3)
            and bits_equal(a.pml, b.pml))


@pytest.mark.parametrize("name", FIXTURES)
def test_golden_runs_bit_exact(emul, name):
    prob, _, d = load_fixture(name)
    rec, mx, st, _ = emul_run(emul, prob)
    assert bits_equal(rec, d["record"]) and bits_equal(mx, d["uxyzmax"])
    assert bits_equal(st.u2, d["u_cur"]) and bits_equal(st.u1, d["u_prev"])


@pytest.mark.parametrize("dims,seed", [((22, 26, 18, 8), 1), ((33, 21, 27, 12), 2),
                                       ((40, 36, 30, 3), 3)])
def test_random_states_bit_exact(emul, dims, seed):
    """Every PML face active and gradients on both sides of the threshold."""
    hx, hy, nz0, pml = dims
    shot = synthetic.small_case(hx=hx, hy=hy, nz0=nz0, pml=pml, nt=4, seed=seed)
    prob = shot.to_oracle(O)
    u_prev, u_cur, pml_state = synthetic.random_state(shot, seed=seed)

    def st():
        s = O.State(prob)
        s.u1[:], s.u2[:], s.u3[:], s.pml[:] = u_prev, u_cur, u_cur, pml_state
        return s

    r32, m32, s32 = O.run(O.REF32, prob, state=st())
    rec, mx, se, cnt = emul_run(emul, prob, state=st())
    assert cnt[0] > 0 and (cnt[1] > 0) == (pml > 5)
    assert bits_equal(mx, m32) and bits_equal(rec, r32) and _same_state(se, s32)


def test_plain_shot_bit_exact(emul):
    """A scaled plain shot (40^3 + 12-cell PML, 300 steps): the wavefield
    fills the grid and crosses every face."""
    shot = synthetic.linear_vti(h=40, nz0=40, pml=12, nt=300, src=(20, 20, 5))
    prob = shot.to_oracle(O)
    r32, m32, s32 = O.run(O.REF32, prob)
    rec, mx, se, _ = emul_run(emul, prob)
    assert bits_equal(mx, m32)
    assert bits_equal(rec, r32)
    assert _same_state(se, s32)


def test_scalar_operator_random(emul):
    """scalar_s against the reference's expression, 4 M random cells with
    gradients over many binades and eps, delta in the configured ranges."""
    rng = np.random.default_rng(11)
    n = 4_000_000
    scale = np.float32(10.0) ** rng.uniform(-6, 2, n).astype(np.float32)
    g = (rng.standard_normal((3, n)) * scale).astype(np.float32)
    # some components exactly zero, some tiny next to the others
    g[0, ::97] = 0.0
    g[1, ::89] *= np.float32(1e-7)
    eps = rng.uniform(0, 0.3, n).astype(np.float32)
    de = (rng.uniform(0, 1, n) * np.minimum(eps, 0.15)).astype(np.float32)
    e2 = (np.float32(2) * eps).astype(np.float32)
    r8 = (np.float32(8) * (eps - de)).astype(np.float32)
    got = np.zeros(n, np.float32)
    want = np.zeros(n, np.float32)
    bad = emul.emul_check_scalar(_p(g[0]), _p(g[1]), _p(g[2]), _p(e2), _p(r8), n, _p(got),
                                 _p(want))
    assert bad == 0, np.nonzero(got.view(np.uint32) != want.view(np.uint32))[0][:10]
    ufb = np.zeros(1, np.int64)
    sfb = np.zeros(1, np.int64)
    emul.emul_fallback_rates(_p(g[0]), _p(g[1]), _p(g[2]), _p(e2), _p(r8), n, _p(ufb), _p(sfb))
    print("FP64 fallbacks per million cells: unit normal %.1f, S %.1f" %
          (1e6 * ufb[0] / n, 1e6 * sfb[0] / n))
    assert ufb[0] < n * 1e-3 and sfb[0] < n * 1e-3
