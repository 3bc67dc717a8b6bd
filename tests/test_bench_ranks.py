"""bench.py's multi-rank contract on the CPU: launched by torch.distributed.run
with two ranks (gloo), the reference arm runs on rank 0 only and prints one
JSON line; the other rank exits 0 without work."""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_reference_arm_two_ranks(tmp_path):
    pytest.importorskip("torch.distributed")
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", "--nproc-per-node=2",
           "--master-addr", "127.0.0.1", "--master-port", "29533",
           os.path.join(ROOT, "bench.py"), "--impl", "reference", "--gpus", "2",
           "--steps", "1", "--warmup", "0", "--scale", "0.1", "--nt", "20"]
    env = dict(os.environ, OMP_NUM_THREADS="2", QP3D_BENCH_BACKEND="gloo")
    r = subprocess.run(cmd, capture_output=True, text=True, timeout=600, cwd=str(tmp_path), env=env)
    assert r.returncode == 0, r.stderr[-2000:]
    lines = [l for l in r.stdout.splitlines() if l.startswith("{")]
    assert len(lines) == 1, r.stdout
    d = json.loads(lines[0])
    assert d["impl"] == "reference" and d["n_gpus"] == 2 and d["value"] > 0
    assert d["cpu_baseline"]["kind"] == "port" and d["e2e"]["h2d_bytes_per_step"] == 0
    # the CPU reference never loads the library it is compared with
    assert d["native_libs"] and all(l.startswith("oracle") for l in d["native_libs"]), d


def test_reference_inputs_match_library_inputs():
    """The oracle backend of the workload generator builds the same inputs
    as the library's host utilities, bit for bit."""
    import numpy as np
    import synthetic
    a = synthetic.small_case(nt=30, seed=5)
    synthetic.set_backend("oracle")
    try:
        b = synthetic.small_case(nt=30, seed=5)
    finally:
        synthetic.set_backend("qp3d")
    assert type(b).__module__.endswith("oracle")
    for x, y in [(a.vp, b.vp), (a.eps, b.eps), (a.delta, b.delta), (a.src, b.src),
                 (a.wavelet, b.wavelet), (a.c, b.c), (a.c2, b.c2)] + list(zip(a.prof, b.prof)):
        assert np.array_equal(np.asarray(x).view(np.uint32), np.asarray(y).view(np.uint32))
    assert (a.nx, a.ny, a.nz, a.pml, a.sz) == (b.nx, b.ny, b.nz, b.pml, b.sz)
