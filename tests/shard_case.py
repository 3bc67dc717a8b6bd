"""Worker of tests/test_shard.py: one gloo rank on the CPU.

Each rank computes the gradient terms of its own block of shots -- either a
deterministic stand-in with a wide dynamic range (so that the order of the
FP64 additions shows in the result), or the oracle's FP64 adjoint of small
shots -- and the records of its block, then takes part in the ordered
gradient sum and the record gather of the shard module.
"""
import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG = os.path.join(ROOT, "gpu-c_3dqmodeling_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402


class FakeShot:
    """Shape of a shot as the shard module sees it."""

    def __init__(self, i, nx=12, ny=10, nz=8, nt=5):
        self.i, self.nx, self.ny, self.nz, self.nt = i, nx + i % 3, ny, nz, nt + i
        self.N = 600
        self.hx, self.hy = 3 + i % 2, 4


def fake_terms(i, n=600):
    """Gradient terms of shot i: magnitudes spread over 2^-30 .. 2^30."""
    rng = np.random.default_rng(100 + i)
    g = [rng.standard_normal(n) * np.exp2(rng.integers(-30, 31, n)) for _ in range(3)]
    return float(rng.random() * 10 ** (i % 5)), g


def fake_record(s):
    rng = np.random.default_rng(7 + s.i)
    return rng.standard_normal((s.nt, s.hx, s.hy)).astype(np.float32)


def oracle_shots(n=3):
    import synthetic
    synthetic.set_backend("oracle")
    shots = [synthetic.small_case(hx=14, hy=12, nz0=10, pml=4, nt=30, seed=60 + i, fm=35.0)
             for i in range(n)]
    return shots


def adding(terms_fn):
    """grad_fn of shard.gradient from a function returning (J, terms)."""
    def fn(i, s, out):
        J, g = terms_fn(i, s)
        for q in range(3):
            out[q] += g[q]
        return J
    return fn


def oracle_terms(i, shot):
    """(misfit, FP64 gradient) of one small shot by the oracle's adjoint, with
    observed data made by scaling its own record."""
    from oracle import oracle as O
    adj = O.Adjoint(shot).freeze()
    rec, hist = adj.forward(want_hist=True)
    d_obs = 0.9 * rec + 1e-3 * (i + 1)
    r = rec - d_obs
    g = adj.backward(hist, r)
    return 0.5 * float(np.sum(r * r)), list(g)


def worker(rank, world, port, kind, out_q):
    import torch.distributed as dist
    import shard
    dist.init_process_group("gloo", init_method="tcp://127.0.0.1:%d" % port, rank=rank,
                            world_size=world)
    try:
        if kind in ("fake", "fake2"):
            shots = [FakeShot(i) for i in range(7)]
            fn = adding(lambda i, s: fake_terms(i))
            J, G = shard.gradient(shots, [fn, fn, fn] if kind == "fake2" else fn)
            blk, recs = shard.records(shots, lambda b: [fake_record(s) for s in b])
        else:
            shots = oracle_shots()
            J, G = shard.gradient(shots, adding(oracle_terms))
            blk, recs = (0, 0), []
        out_q.put((rank, J, [g.copy() for g in G], blk, [r.copy() for r in recs]))
    finally:
        dist.destroy_process_group()
