"""The FP64 adjoint of the oracle (the checker of qp3d_adjoint), on the CPU.

* dot-product test: the adjoint propagation is the exact transpose of the
  frozen-operator forward, PML recursions included:
  <P f, r> = <f, P^T r> for random additive sources f and record residuals r;
  and with the live operator, the exact transpose of the tangent-linear run
  about the base trajectory (S perturbed through the unit normal);
* finite differences: the adjoint-state gradient of 1/2 |R u - d|^2 with
  respect to vp, eps and delta on the cells outside the PML shell matches
  central differences of the frozen-operator forward;
* with the live operator (S's dependence on grad u differentiated as well)
  it matches central differences of the live forward, the scalar operator
  recomputed from each perturbed wavefield.
"""
import numpy as np
import pytest

import synthetic
from oracle import oracle as O


def _problem(nt=60, pml=6, seed=41):
    shot = synthetic.small_case(hx=18, hy=16, nz0=14, pml=pml, nt=nt, seed=seed, fm=35.0)
    return shot.to_oracle(O)


@pytest.mark.parametrize("pml", [6, 0])
def test_adjoint_dot_product(pml):
    prob = _problem(nt=50, pml=pml)
    adj = O.Adjoint(prob, source=False).freeze(with_source=True)
    rng = np.random.default_rng(3)
    extra = rng.standard_normal((prob.nt, prob.N)) * (rng.random((prob.nt, prob.N)) < 0.02)
    rec, hist = adj.forward(extra=extra, want_hist=True)
    r = rng.standard_normal(rec.shape)
    _, fadj = adj.backward(hist, r, want_fadj=True)
    lhs = float(np.dot(rec.ravel(), r.ravel()))
    rhs = float(np.dot(extra.ravel(), fadj))
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_live_adjoint_dot_product():
    """<L f, r> = <f, L^T r> for the tangent-linear run of the live operator
    (measured to 3e-15), whose records differ from the frozen operator's."""
    prob = _problem(nt=50, pml=6)
    out = {}
    for live in (True, False):
        adj = O.Adjoint(prob, live=live).freeze()
        _, hist = adj.forward(want_hist=True)
        rng = np.random.default_rng(3)
        extra = rng.standard_normal((prob.nt, prob.N)) * (rng.random((prob.nt, prob.N)) < 0.02)
        rec = adj.tlm(hist, extra)
        r = rng.standard_normal(rec.shape)
        _, fadj = adj.backward(hist, r, want_fadj=True)
        lhs = float(np.dot(rec.ravel(), r.ravel()))
        rhs = float(np.dot(extra.ravel(), fadj))
        assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (live, lhs, rhs)
        out[live] = lhs
    assert abs(out[True] - out[False]) > 1e-4 * abs(out[False])


def _interior_mask(prob):
    m = np.zeros((prob.nz, prob.nx, prob.ny), bool)
    p = prob.pml
    m[p:prob.nz - p, p:prob.nx - p, p:prob.ny - p] = True
    return m.ravel()


@pytest.mark.parametrize("param", ["vp", "eps", "delta"])
def test_adjoint_gradient_finite_differences(param):
    prob = _problem(nt=60)
    adj = O.Adjoint(prob).freeze()
    # observed data: a smooth perturbation of the model
    rng = np.random.default_rng(7)
    inside = _interior_mask(prob)
    z, x, y = np.meshgrid(np.arange(prob.nz), np.arange(prob.nx), np.arange(prob.ny),
                          indexing="ij")
    blob = np.exp(-(((z - prob.nz / 2) / 4.0) ** 2 + ((x - prob.nx / 2) / 4.0) ** 2 +
                    ((y - prob.ny / 2) / 4.0) ** 2)).ravel() * inside
    d_obs = adj.forward(vp=adj.vp * (1 + 0.03 * blob))
    rec, hist = adj.forward(want_hist=True)
    g_vp, g_eps, g_del = adj.backward(hist, rec - d_obs)
    g = {"vp": g_vp, "eps": g_eps, "delta": g_del}[param]
    base = {"vp": adj.vp, "eps": adj.eps, "delta": adj.delta}[param]
    dm = rng.standard_normal(prob.N) * inside * (np.abs(base).max() if param == "vp" else 0.1)

    def J(h):
        kw = {param: base + h * dm}
        return 0.5 * float(np.sum((adj.forward(**kw) - d_obs) ** 2))

    h = 1e-4 if param == "vp" else 1e-3
    fd = (J(h) - J(-h)) / (2 * h)
    an = float(np.dot(g, dm))
    assert abs(fd - an) <= 1e-5 * abs(fd), (param, fd, an)
    assert np.all(g[~inside] == 0)


@pytest.mark.parametrize("param", ["vp", "eps", "delta"])
def test_live_adjoint_gradient_finite_differences(param):
    prob = _problem(nt=60)
    adj = O.Adjoint(prob, live=True).freeze()
    rng = np.random.default_rng(7)
    inside = _interior_mask(prob)
    z, x, y = np.meshgrid(np.arange(prob.nz), np.arange(prob.nx), np.arange(prob.ny),
                          indexing="ij")
    blob = np.exp(-(((z - prob.nz / 2) / 4.0) ** 2 + ((x - prob.nx / 2) / 4.0) ** 2 +
                    ((y - prob.ny / 2) / 4.0) ** 2)).ravel() * inside
    d_obs = adj.live_forward(vp=adj.vp * (1 + 0.03 * blob))
    rec, hist = adj.forward(want_hist=True)
    g_vp, g_eps, g_del = adj.backward(hist, rec - d_obs)
    g = {"vp": g_vp, "eps": g_eps, "delta": g_del}[param]
    base = {"vp": adj.vp, "eps": adj.eps, "delta": adj.delta}[param]
    dm = rng.standard_normal(prob.N) * inside * (np.abs(base).max() if param == "vp" else 0.1)

    def J(h):
        r = adj.live_forward(**{param: base + h * dm}) - d_obs
        return 0.5 * float(np.sum(r * r))

    h = 1e-5 if param == "vp" else 1e-4
    fd = (J(h) - J(-h)) / (2 * h)
    an = float(np.dot(g, dm))
    # measured 4e-8 (vp), 2e-9 (eps), 8e-9 (delta); the frozen operator's
    # gradient is 1.4e-4, 1.1e-4 and 1.1e-1 away from the same differences
    assert abs(fd - an) <= 1e-6 * abs(fd), (param, fd, an)
    assert np.all(g[~inside] == 0)
