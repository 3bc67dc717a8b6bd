"""qp3d_adjoint: gradient of the record misfit in vp, epsilon and delta.

Checked against the FP64 oracle adjoint of the same step (itself checked by
dot-product and finite-difference tests, test_adjoint_oracle.py): cosine >=
0.999 per parameter with FP32 and with BF16 checkpoints, and with every u^k
kept (bit-identical to FP32 checkpoints), for the live operator (the
default: S's dependence on grad u included) and for S frozen
("adj_live" = 0).  The live gradient agrees with central differences of the
live forward (the scalar operator recomputed from the perturbed wavefield)
to 1 %; the frozen one does not.
"""
import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


def _case(nt=120):
    shot = synthetic.small_case(hx=22, hy=20, nz0=18, pml=8, nt=nt, seed=51, fm=30.0)
    nz, nx, ny = shot.nz, shot.nx, shot.ny
    inside = np.zeros((nz, nx, ny), bool)
    p = shot.pml
    inside[p:nz - p, p:nx - p, p:ny - p] = True
    z, x, y = np.meshgrid(np.arange(nz), np.arange(nx), np.arange(ny), indexing="ij")
    blob = np.exp(-(((z - nz / 2) / 4.0) ** 2 + ((x - nx / 2) / 5.0) ** 2 +
                    ((y - ny / 2) / 5.0) ** 2)) * inside
    true = qp3d.Shot(shot.nx, shot.ny, shot.nz, shot.pml, shot.sz, shot.dx, shot.dy, shot.dz,
                     shot.dt, shot.vp * (1 + 0.04 * blob.ravel()).astype(np.float32),
                     shot.eps, shot.delta, shot.src, shot.wavelet, shot.prof, shot.c, shot.c2)
    return shot, true, inside.ravel()


def _cos(a, b):
    return float(np.dot(a, b) / (np.linalg.norm(a) * np.linalg.norm(b)))


@pytest.fixture(scope="module")
def reference():
    shot, true, inside = _case()
    with qp3d.Context(0) as ctx:
        d_obs = ctx.forward(true)
    prob = shot.to_oracle(O)
    g64 = {}
    for live in (1, 0):
        adj = O.Adjoint(prob, live=bool(live)).freeze()
        rec, hist = adj.forward(want_hist=True)
        g64[live] = adj.backward(hist, rec - d_obs.astype(np.float64))
    J64 = 0.5 * float(np.sum((rec - d_obs) ** 2))
    return shot, d_obs, g64, J64, inside


@pytest.mark.parametrize("bf16,keep,live", [(0, 0, 1), (1, 0, 1), (0, 1, 1), (0, 0, 0),
                                            (1, 0, 0), (0, 1, 0)])
def test_adjoint_gradient_matches_fp64(reference, bf16, keep, live):
    shot, d_obs, g64s, J64, inside = reference
    g64 = g64s[live]
    with qp3d.Context(0) as ctx:
        assert ctx.tuning("adj_live") == 1            # the default
        ctx.tune(adj_ckpt_bf16=bf16, adj_keep_all=keep, adj_live=live)
        J, g = ctx.adjoint(shot, d_obs)
        J2, g2 = ctx.adjoint(shot, d_obs)     # buffers reused: same result
    assert abs(J - J64) <= 1e-4 * J64, (J, J64)
    label = ("live " if live else "frozen ") + (
        "keep all" if keep else "ckpt " + ("bf16" if bf16 else "fp32"))
    for name, gi, ri in zip(("vp", "eps", "delta"), g, g64):
        c = _cos(gi, ri)
        print("%s %s: cosine vs FP64 adjoint %.6f" % (label, name, c))
        assert c >= 0.999, (name, c)
        assert np.all(gi[~inside] == 0)
    for a, b in zip(g, g2):
        assert np.array_equal(a, b)


def test_adjoint_schedules_agree(reference):
    # keeping every u^k and recomputing from FP32 checkpoints run the same
    # adjoint steps on the same wavefields: identical gradients
    shot, d_obs, _, _, _ = reference
    out = []
    for keep in (0, 1, -1):
        with qp3d.Context(0) as ctx:
            ctx.tune(adj_ckpt_bf16=0, adj_keep_all=keep)
            out.append(ctx.adjoint(shot, d_obs))
    for J, g in out[1:]:
        # the misfit is an FP64 sum of per-block atomics: order-dependent
        assert J == pytest.approx(out[0][0], rel=1e-12)
        for a, b in zip(g, out[0][1]):
            assert np.array_equal(a, b)


def test_adjoint_without_steps():
    shot = synthetic.small_case(hx=16, hy=14, nz0=12, pml=6, nt=0, seed=52)
    with qp3d.Context(0) as ctx:
        J, g = ctx.adjoint(shot, np.zeros((0, shot.hx, shot.hy), np.float32))
    assert J == 0.0
    assert all(not np.any(gi) for gi in g)


@pytest.mark.parametrize("live", [1, 0])
def test_adjoint_against_live_finite_differences(reference, live):
    """The vp gradient against central differences of the live forward (S
    recomputed from each perturbed wavefield): of the scheme in FP64 (the
    oracle, h = 0.02 m/s, where the differences have converged to 1e-9) and of
    the library's FP32 forward (h = 0.2 m/s; at 2 m/s threshold flips and
    curvature move the difference by 2.5 %)."""
    shot, d_obs, _, _, inside = reference
    rng = np.random.default_rng(11)
    dm = (rng.standard_normal(shot.N) * inside).astype(np.float64)
    with qp3d.Context(0) as ctx:
        ctx.tune(adj_ckpt_bf16=0, adj_live=live)
        _, g = ctx.adjoint(shot, d_obs)

        def J(h):
            s = qp3d.Shot(shot.nx, shot.ny, shot.nz, shot.pml, shot.sz, shot.dx, shot.dy,
                          shot.dz, shot.dt, (shot.vp + h * dm).astype(np.float32), shot.eps,
                          shot.delta, shot.src, shot.wavelet, shot.prof, shot.c, shot.c2)
            r = ctx.forward(s).astype(np.float64) - d_obs
            return 0.5 * float(np.sum(r * r))

        fd32 = (J(0.2) - J(-0.2)) / 0.4
    adj = O.Adjoint(shot.to_oracle(O), live=True)
    vp64 = shot.vp.astype(np.float64)

    def J64(h):
        r = adj.live_forward(vp=vp64 + h * dm) - d_obs
        return 0.5 * float(np.sum(r * r))

    fd64 = (J64(0.02) - J64(-0.02)) / 0.04
    an = float(np.dot(g[0], dm))
    print("vp, %s operator: adjoint %.7e, central differences of the live forward: FP64 "
          "scheme %.7e (rel %.2e), FP32 library %.7e (rel %.2e)"
          % ("live" if live else "frozen", an, fd64, abs(an - fd64) / abs(fd64), fd32,
             abs(an - fd32) / abs(fd32)))
    if live:
        assert abs(an - fd64) <= 1e-4 * abs(fd64)
        assert abs(an - fd32) <= 0.01 * abs(fd32)
    else:
        # the frozen operator leaves out dS/du (7 % on this case)
        assert 0.01 * abs(fd64) <= abs(an - fd64) <= 0.15 * abs(fd64)


def test_bf16_checkpoints_at_reduced_gradient_workload():
    """The gradient workload at reduced size (the 12-layer model of the
    16-shot case at 100x100x75 cells + 20-cell PML, a start model smoothed
    by sigma = 2.5 cells, 2x2 shots, 800 steps): sqrt(nt) checkpoints with the
    PML levels in BF16 and the forward's threshold decisions replayed, against
    every u^k kept in FP32 (the schedule checked against the FP64 adjoint
    above): cosine >= 0.999 for vp, eps and delta."""
    true, start = synthetic.adjoint_case(hx=100, hy=100, nz0=75, pml=20, nt=800, sigma=2.5,
                                         grid=2)
    out = {}
    with qp3d.Context(0) as ctx:
        assert ctx.tuning("adj_ckpt_bf16") == 1      # the default storage
        d_obs = [ctx.forward(s).copy() for s in true]
        for name, bf16, keep in (("bf16", 1, 0), ("fp32", 0, 0), ("keep", 0, 1)):
            ctx.tune(adj_ckpt_bf16=bf16, adj_keep_all=keep)
            grads = [np.zeros(start[0].N, np.float64) for _ in range(3)]
            for s, d in zip(start, d_obs):
                ctx.adjoint(s, d, grads)
            out[name] = grads
    for a, b in zip(out["fp32"], out["keep"]):
        assert np.array_equal(a, b)
    for name, a, b in zip(("vp", "eps", "delta"), out["bf16"], out["keep"]):
        c = _cos(a, b)
        print("reduced gradient workload, BF16 PML checkpoints %s: cosine %.6f" % (name, c))
        assert c >= 0.999, (name, c)


def test_gradient_on_two_contexts_equals_one():
    """shard.gradient with two library contexts on the GPU (two shots at a
    time, each on its own stream and host thread) adds the shots' terms in
    shot order: bit for bit the gradient of one context taking the shots in
    turn, keeping every u^k and with BF16 checkpoints."""
    import shard
    shots, d_obs = [], []
    with qp3d.Context(0) as ctx:
        for seed in (51, 52, 53, 54):
            s = synthetic.small_case(hx=22, hy=20, nz0=18, pml=8, nt=80, seed=seed, fm=30.0)
            true = qp3d.Shot(s.nx, s.ny, s.nz, s.pml, s.sz, s.dx, s.dy, s.dz, s.dt,
                             (s.vp * np.float32(1.02)).astype(np.float32), s.eps, s.delta, s.src,
                             s.wavelet, s.prof, s.c, s.c2)
            shots.append(s)
            d_obs.append(ctx.forward(true).copy())
    N = shots[0].N
    for keep in (1, 0):
        with qp3d.Context(0) as c0, qp3d.Context(0) as c1:
            for c in (c0, c1):
                c.tune(adj_keep_all=keep)
            one = [np.zeros(N, np.float64) for _ in range(3)]
            J1 = 0.0
            for s, d in zip(shots, d_obs):
                J1 += c0.adjoint(s, d, one)[0]
            fns = [lambda i, s, out, c=c: c.adjoint(s, d_obs[i], out)[0] for c in (c0, c1)]
            J2, two = shard.gradient(shots, fns, group=shard.Group())
        assert J2 == pytest.approx(J1, rel=1e-12)
        for a, b in zip(one, two):
            assert np.array_equal(a.view(np.uint64), b.view(np.uint64))
