"""Helpers shared by the test modules (fixture loading, error metrics)."""
import os

import numpy as np

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
FIXTURES = ["layered_small", "pml5_wide_source"]


def load_fixture(name):
    """(oracle Problem, library Shot, expected outputs) of a golden fixture."""
    from oracle import oracle as O
    import qp3d
    d = np.load(os.path.join(GOLDEN, name + ".npz"))
    nx, ny, nz, pml, sz = [int(v) for v in d["geom"]]
    dx, dy, dz, dt = [float(v) for v in d["spacing"]]
    args = (nx, ny, nz, pml, sz, dx, dy, dz, dt, d["vp"], d["eps"], d["delta"], d["source"],
            d["wavelet"], list(d["prof"]), d["c"], d["c2"])
    return O.Problem(*args), qp3d.Shot(*args), d


def rel_l2(a, b):
    a = np.asarray(a, np.float64).ravel()
    b = np.asarray(b, np.float64).ravel()
    n = np.linalg.norm(b)
    return float(np.linalg.norm(a - b) / n) if n > 0 else float(np.linalg.norm(a - b))


def max_abs_rel_peak(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    p = np.abs(b).max()
    return float(np.abs(a - b).max() / p) if p > 0 else float(np.abs(a - b).max())


def bits_equal(a, b):
    a = np.ascontiguousarray(a, np.float32)
    b = np.ascontiguousarray(b, np.float32)
    return a.shape == b.shape and np.array_equal(a.view(np.uint32), b.view(np.uint32))


_PLAIN = {}


def plain_shot_oracles(shot):
    """(REF32 record, FP64 record) of a whole shot, computed once per test
    session for a given shot geometry and model (the 1000-step plain shot is
    compared in several tests)."""
    from oracle import oracle as O
    key = (shot.nx, shot.ny, shot.nz, shot.pml, shot.nt, shot.sz,
           float(np.asarray(shot.vp, np.float64).sum()), float(np.asarray(shot.eps).sum()))
    if key not in _PLAIN:
        prob = shot.to_oracle(O)
        r32, _, _ = O.run(O.REF32, prob)
        r64, _, _ = O.run(O.F64, prob)
        _PLAIN[key] = (r32, r64)
    return _PLAIN[key]
