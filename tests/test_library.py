"""libqp3d.so host-side checks that need no GPU.

The library must load without a GPU driver, export every symbol the public
headers declare, and its host utilities must reproduce the reference's
(CPU_function.c) bit for bit -- checked against the oracle, which is pinned
to the reference by test_oracle.py.
"""
import ctypes
import os
import re
import subprocess

import numpy as np
import pytest

import qp3d
from oracle import oracle as O
from helpers import bits_equal, load_fixture

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared_symbols():
    names = set()
    for h in ("qp3d.h", "qp3d_driver.h"):
        text = open(os.path.join(ROOT, "include", h)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(qp3d_[a-z0-9_]+)\s*\(", text):
            names.add(m.group(1))
    return names


def test_exports_every_declared_symbol():
    lib = qp3d.load()
    declared = _declared_symbols()
    assert declared, "no declarations parsed"
    assert declared <= set(qp3d.EXPORTS), declared - set(qp3d.EXPORTS)
    for name in declared:
        assert hasattr(lib, name), name
    out = subprocess.run(["nm", "-D", "--defined-only", qp3d.LIB_PATH], capture_output=True,
                         text=True).stdout
    assert re.search(r"\bT _Z10modeling3d", out), "C++-linkage modeling3d drop-in missing"


def test_no_runtime_dependency_on_cuda_driver():
    out = subprocess.run(["ldd", qp3d.LIB_PATH], capture_output=True, text=True).stdout
    assert "libcuda.so" not in out and "libcudart.so" not in out


def test_fdcoff_matches_oracle():
    c, c2 = qp3d.fdcoff()
    oc, oc2 = O.fdcoff()
    assert bits_equal(c, oc) and bits_equal(c2, oc2)


@pytest.mark.parametrize("pml,vpmax,dx,dy,dz", [(20, 4900.0, 10.0, 10.0, 10.0),
                                                (30, 6300.0, 12.5, 10.0, 8.0), (5, 3000.0, 5.0, 5.0, 5.0)])
def test_pmlcoff_matches_oracle(pml, vpmax, dx, dy, dz):
    a = qp3d.pmlcoff(pml, vpmax, dx, dy, dz)
    b = O.pmlcoff(pml, vpmax, dx, dy, dz)
    for x, y in zip(a, b):
        assert bits_equal(x, y)


@pytest.mark.parametrize("alpha", [1.0, 0.05])
def test_source_matches_oracle(alpha):
    args = (9, 11, 7, 25.0, 1.0, alpha, 5e-4, 10.0, 10.0, 10.0, 1.0 / 25.0, 300, 21, 23, 19)
    s1, w1 = qp3d.source(*args)
    s2, w2 = O.source(*args)
    assert bits_equal(s1, s2)
    assert bits_equal(w1, w2)


def test_extend_model_matches_oracle():
    rng = np.random.default_rng(3)
    interior = rng.standard_normal((9, 13, 11)).astype(np.float32)
    pml = 6
    a = qp3d.extend_model(interior, 13 + 2 * pml, 11 + 2 * pml, 9 + 2 * pml, pml)
    b = O.extend_model(interior, 13 + 2 * pml, 11 + 2 * pml, 9 + 2 * pml, pml)
    assert bits_equal(a, b)


def test_absmax_semantics():
    a = np.array([0.0, -3.0, 2.0, np.nan, -3.0], np.float32)
    assert qp3d.absmax(a) == 3.0
    assert qp3d.absmax(np.zeros(4, np.float32)) == 0.0


def test_readmodel3d_window(tmp_path):
    """File [vny][vnx][vnz] (z fastest, model/grey3_tmp.rsf) -> a[nz][nx][ny]."""
    vny, vnx, vnz = 7, 6, 5
    data = np.arange(vny * vnx * vnz, dtype=np.float32).reshape(vny, vnx, vnz)
    f = tmp_path / "m.dat"
    data.tofile(f)
    ny, nx, nz, fny, fnx, fnz = 3, 4, 2, 2, 1, 3
    out = np.zeros(nz * nx * ny, np.float32)
    rc = qp3d.load().qp3d_readmodel3d(str(f).encode(), out.ctypes.data_as(ctypes.c_void_p),
                                      ny, nx, nz, fny, fnx, fnz, vny, vnx, vnz)
    assert rc == 0
    want = data[fny:fny + ny, fnx:fnx + nx, fnz:fnz + nz].transpose(2, 1, 0)
    assert np.array_equal(out.reshape(nz, nx, ny), want)
    # missing file and a window past the end are errors, not silent garbage
    assert qp3d.load().qp3d_readmodel3d(str(tmp_path / "nope.dat").encode(),
                                        out.ctypes.data_as(ctypes.c_void_p),
                                        ny, nx, nz, 0, 0, 0, vny, vnx, vnz) == -6
    assert qp3d.load().qp3d_readmodel3d(str(f).encode(), out.ctypes.data_as(ctypes.c_void_p),
                                        ny, nx, nz, 5, 0, 0, vny, vnx, vnz) == -1


def test_pml_state_size_matches_oracle():
    for g in [(40, 44, 38, 10), (140, 140, 140, 20), (31, 37, 29, 0)]:
        assert qp3d.pml_state_size(*g) == O.pml_state_size(*g)


def test_synthetic_generators_are_deterministic():
    import synthetic
    a = synthetic.small_case(seed=5)
    b = synthetic.small_case(seed=5)
    assert bits_equal(a.vp, b.vp) and bits_equal(a.eps, b.eps) and bits_equal(a.src, b.src)
    c = synthetic.small_case(seed=6)
    assert not bits_equal(a.vp, c.vp)
    assert a.nt == 60 and a.nx == 22 + 16


def test_context_without_device_fails_cleanly():
    try:
        import torch
        has_gpu = torch.cuda.is_available()
    except Exception:
        has_gpu = os.path.exists("/dev/nvidia0")
    if has_gpu:
        pytest.skip("a GPU is present")
    with pytest.raises(qp3d.QP3DError):
        qp3d.Context(0)


def test_reference_program_links_against_the_library(tmp_path):
    """Link-time drop-in: the reference's own main program, compiled from its
    unmodified sources in the reference checkout (outputs in tmp_path), links
    against libqp3d.so with modeling3d resolved from the library; and a C
    program using only include/qp3d.h compiles as C99 and links."""
    from oracle import build as ob
    if not ob.reference_available():
        pytest.skip("reference checkout not present")
    lib_dir = os.path.dirname(qp3d.LIB_PATH)
    objs = []
    for src in ("array_new.c", "read_write.c", "CPU_function.c", "3dPureqPModeling1.0.c"):
        o = str(tmp_path / (src[:-2] + ".o"))
        # the reference compiles its .c files as C++ (Makefile:9)
        r = subprocess.run(["g++", "-w", "-c", "-I", ob.REFERENCE_DIR,
                            os.path.join(ob.REFERENCE_DIR, src), "-o", o],
                           capture_output=True, text=True)
        assert r.returncode == 0, r.stderr
        objs.append(o)
    exe = str(tmp_path / "3dqpmodeling")
    r = subprocess.run(["g++", "-o", exe] + objs + ["-L" + lib_dir, "-lqp3d",
                                                    "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    undefined = subprocess.run(["nm", "-C", "--undefined-only", exe], capture_output=True,
                               text=True).stdout
    assert "modeling3d(int, int, int" in undefined        # provided by libqp3d.so
    defined = subprocess.run(["nm", "-C", "-D", "--defined-only", qp3d.LIB_PATH],
                             capture_output=True, text=True).stdout
    assert "modeling3d(int, int, int" in defined


def test_c_program_against_the_public_header(tmp_path):
    src = tmp_path / "use_abi.c"
    src.write_text('''
#include <stdio.h>
#include "qp3d.h"
#include "qp3d_driver.h"
int main(void)
{
    qp3d_ctx *ctx = NULL;
    int rc = qp3d_ctx_create(0, &ctx);
    printf("%d %s\\n", rc, qp3d_strerror(rc));
    if (rc == QP3D_OK) qp3d_ctx_destroy(ctx);
    return 0;
}
''')
    lib_dir = os.path.dirname(qp3d.LIB_PATH)
    exe = str(tmp_path / "use_abi")
    r = subprocess.run(["gcc", "-std=c99", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                        str(src), "-o", exe, "-L" + lib_dir, "-lqp3d", "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0
    rc = int(out.stdout.split()[0])
    assert rc in (0, -2)   # QP3D_OK on a GPU machine, QP3D_ERR_CUDA without one


def test_source_scan_matches_a_sequential_scan(tmp_path):
    """The threaded scan of the source volume (qp3d::scan_source_volume, used
    by qp3d_shot_load and qp3d_batch) returns every non-zero sample in the
    order of one sequential z, x, y scan."""
    src = tmp_path / "scan.cpp"
    src.write_text(r'''
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "qp3d_internal.h"
int main()
{
    const int nx = 37, ny = 29, nz = 53;
    std::vector<float> v((size_t)nx * ny * nz, 0.0f);
    unsigned s = 12345u;
    for (size_t i = 0; i < v.size(); ++i) {
        s = s * 1664525u + 1013904223u;
        if ((s >> 24) < 3) v[i] = (float)(s & 0xffff) - 30000.0f;   /* ~1% non-zero */
    }
    std::vector<qp3d::SrcEntry> got;
    qp3d::scan_source_volume(v.data(), nx, ny, nz, got);
    size_t k = 0;
    for (int z = 0; z < nz; ++z)
        for (int x = 0; x < nx; ++x)
            for (int y = 0; y < ny; ++y) {
                const float f = v[((size_t)z * nx + x) * ny + y];
                if (f == 0.0f) continue;
                if (k >= got.size() || got[k].x != x || got[k].y != y || got[k].z != z ||
                    got[k].v != f) {
                    printf("mismatch at %zu\n", k);
                    return 1;
                }
                ++k;
            }
    printf("%zu %zu\n", k, got.size());
    return k == got.size() ? 0 : 1;
}
''')
    lib_dir = os.path.dirname(qp3d.LIB_PATH)
    exe = str(tmp_path / "scan")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "gpu-c_3dqmodeling_gb300",
                                                                     "csrc"),
                        "-I", os.path.join(ROOT, "include"), "-I", "/usr/local/cuda/include",
                        str(src), "-o", exe, "-L" + lib_dir, "-lqp3d", "-Wl,-rpath," + lib_dir],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    out = subprocess.run([exe], capture_output=True, text=True, timeout=120)
    assert out.returncode == 0, out.stdout
    n, m = (int(t) for t in out.stdout.split())
    assert n == m and n > 100
