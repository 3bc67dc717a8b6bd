"""The CPU oracle against the reference (CPU only).

The oracle's FP32 variant restates the reference operators of
CPU_function.c:301-480; here it is pinned bit for bit to the golden vectors
produced by the reference's own compiled code, and -- where the reference
checkout is present -- to that code directly on further cases.
"""
import numpy as np
import pytest

from oracle import oracle as O
from helpers import FIXTURES, bits_equal, load_fixture, rel_l2


@pytest.mark.parametrize("name", FIXTURES)
def test_ref32_matches_golden_bit_exact(name):
    prob, _, d = load_fixture(name)
    rec, mx, st = O.run(O.REF32, prob)
    assert bits_equal(rec, d["record"])
    assert bits_equal(mx, d["uxyzmax"])
    assert bits_equal(st.u1, d["u_prev"])
    assert bits_equal(st.u2, d["u_cur"])
    assert bits_equal(st.pml, d["pml_state"])


@pytest.mark.parametrize("name", FIXTURES)
def test_host_utilities_match_golden_inputs(name):
    """fdcoff1/2, pmlcoff, Source and extend_model restated in the oracle
    reproduce the inputs the reference made for the fixture."""
    prob, _, d = load_fixture(name)
    c, c2 = O.fdcoff()
    assert bits_equal(c, d["c"]) and bits_equal(c2, d["c2"])
    prof = O.pmlcoff(prob.pml, float(d["vpmax"]), prob.dx, prob.dy, prob.dz)
    assert bits_equal(np.stack(prof), d["prof"])
    for key, vol in (("vp_interior", "vp"), ("eps_interior", "eps"), ("del_interior", "delta")):
        ext = O.extend_model(d[key], prob.nx, prob.ny, prob.nz, prob.pml)
        assert bits_equal(ext, d[vol])
    # the fixture's source is centred where the argmax is
    src = d["source"].reshape(prob.nz, prob.nx, prob.ny)
    z, x, y = np.unravel_index(np.argmax(src), src.shape)
    fm = None
    for cand in (30.0, 35.0):
        _, w = O.source(x, y, z, cand, 1.0, 1.0, prob.dt, prob.dx, prob.dy, prob.dz,
                        1.0 / cand, prob.nt, 11, 11, 11)
        if bits_equal(w, d["wavelet"]):
            fm = cand
    assert fm is not None, "wavelet not reproduced"


def _random_problem(seed, nx=31, ny=37, nz=29, pml=7, nt=6):
    rng = np.random.default_rng(seed)
    N = nx * ny * nz
    vp = rng.uniform(1500, 4500, N).astype(np.float32)
    eps = rng.uniform(0, 0.3, N).astype(np.float32)
    dl = (eps * rng.uniform(0, 0.5, N)).astype(np.float32)
    prof = O.pmlcoff(pml, float(1.6 * 4500), 10.0, 10.0, 10.0)
    c, c2 = O.fdcoff()
    src = np.zeros(N, np.float32)
    src[rng.integers(0, N, 5)] = rng.standard_normal(5).astype(np.float32)
    wav = rng.standard_normal(nt).astype(np.float32)
    return O.Problem(nx, ny, nz, pml, pml + 2, 10.0, 10.0, 10.0, 5e-4, vp, eps, dl, src, wav,
                     prof, c, c2)


def _random_state(prob, seed):
    rng = np.random.default_rng(seed)
    st = O.State(prob)
    st.u1[:] = (1e-3 * rng.standard_normal(prob.N)).astype(np.float32)
    st.u2[:] = (1e-3 * rng.standard_normal(prob.N)).astype(np.float32)
    st.u3[:] = (1e-3 * rng.standard_normal(prob.N)).astype(np.float32)
    st.pml[:] = (1e-3 * rng.standard_normal(st.pml.size)).astype(np.float32)
    return st


@pytest.mark.skipif(O.ref_lib() is None, reason="reference checkout not present")
@pytest.mark.parametrize("seed", [1, 2])
def test_ref32_matches_reference_from_random_state(seed):
    """Every PML face and the interior active from step 0 (random state)."""
    prob = _random_problem(seed)
    s0 = _random_state(prob, seed + 100)
    a = s0.copy()
    b = s0.copy()
    ra, ma, _ = O.run(O.REF32, prob, state=a)
    rb, mb, _ = O.run_reference(prob, state=b)
    assert bits_equal(ra, rb) and bits_equal(ma, mb)
    for k in ("u1", "u2", "u3", "pml"):
        assert bits_equal(getattr(a, k), getattr(b, k)), k


def test_variants_agree_on_a_short_run():
    """Mirror and FP64 stay within FP32 rounding of the reference arithmetic
    before threshold flips accumulate."""
    prob, _, d = load_fixture("layered_small")
    rm, mm, _ = O.run(O.MIRROR, prob)
    r64, m64, _ = O.run(O.F64, prob)
    assert rel_l2(rm, d["record"]) < 1e-5
    assert rel_l2(d["record"], r64) < 1e-5
    assert np.allclose(mm, m64, rtol=1e-5, atol=0)


def test_threshold_helpers():
    for m in [0.0, 1e-30, 3.7e-5, 1.0, 12345.678, np.float32(0.1)]:
        t = O.threshold_f(m)
        assert np.float64(np.float32(t)) <= 1e-2 * np.float64(np.float32(m))
        nxt = np.nextafter(np.float32(t), np.float32(np.inf))
        assert np.float64(nxt) > 1e-2 * np.float64(np.float32(m))
        t2 = np.float32(O.threshold_m2(m))
        assert np.sqrt(t2, dtype=np.float32) <= np.float32(t)
        assert np.sqrt(np.nextafter(t2, np.float32(np.inf)), dtype=np.float32) > np.float32(t)
