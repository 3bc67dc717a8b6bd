"""The C++-linkage modeling3d drop-in (3dPureqPModeling_single_shot.h:4-6),
called through its mangled symbol exactly as the reference's main program
calls it: host buffers in, record out, snapshot files written under the
given prefix.  The record must equal the oracle mirror bit for bit and the
snapshot files must equal the state of the same shot run step by step."""
import ctypes
import os

import numpy as np
import pytest

import qp3d
import synthetic
from oracle import oracle as O
from helpers import bits_equal

pytestmark = pytest.mark.gpu

_MANGLED = "_Z10modeling3diiiiiffffiiiiiPfS_S_S_S_S_S_S_S_S_S_S_S_S_PKc"


def _modeling3d():
    f = getattr(ctypes.CDLL(qp3d.LIB_PATH), _MANGLED)
    i, fl, p = ctypes.c_int, ctypes.c_float, ctypes.c_void_p
    f.argtypes = [i] * 5 + [fl] * 4 + [i] * 5 + [p] * 14 + [ctypes.c_char_p]
    f.restype = None
    return f


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_modeling3d_drop_in(tmp_path):
    shot = synthetic.small_case(hx=22, hy=26, nz0=18, pml=8, nt=45, seed=41)
    ntsnap = 20
    rec = np.full((shot.nt, shot.hx, shot.hy), np.nan, np.float32)
    prefix = str(tmp_path / "snap")
    keep = []   # the arrays must outlive the call

    def arr(a):
        a = np.ascontiguousarray(a, np.float32)
        keep.append(a)
        return _ptr(a)

    _modeling3d()(shot.nx, shot.ny, shot.nz, shot.nt, ntsnap, shot.dx, shot.dy, shot.dz,
                  shot.dt, shot.pml, 1, 0, 0, shot.sz, arr(shot.vp), arr(shot.eps),
                  arr(shot.delta), arr(shot.src), arr(shot.wavelet), _ptr(rec),
                  *[arr(pr) for pr in shot.prof], arr(shot.c), arr(shot.c2), prefix.encode())
    mrec, _, _ = O.run(O.MIRROR, shot.to_oracle(O))
    assert bits_equal(rec, mrec)
    # snapshots at k = 0, 20, 40: the interior volume and its three mid slices
    pml, hx, hy, hz = shot.pml, shot.hx, shot.hy, shot.nz - 2 * shot.pml
    st, done = None, 0
    for k in (0, 20, 40):
        _, _, st = O.run(O.MIRROR, shot.to_oracle(O), k0=done, nsteps=k + 1 - done, state=st,
                         want_record=False)
        done = k + 1
        u = st.u2.reshape(shot.nz, shot.nx, shot.ny)[pml:pml + hz, pml:pml + hx, pml:pml + hy]
        vol = np.fromfile("%s%d.dat" % (prefix, k), np.float32)
        assert bits_equal(vol, u.ravel()), k
        xz = np.fromfile("%s_xz%d.dat" % (prefix, k), np.float32)
        assert bits_equal(xz, u[:, :, (hy - 1) // 2].ravel())
        yz = np.fromfile("%s_yz%d.dat" % (prefix, k), np.float32)
        assert bits_equal(yz, u[:, (hx - 1) // 2, :].ravel())
        xy = np.fromfile("%s_xy%d.dat" % (prefix, k), np.float32)
        assert bits_equal(xy, u[(hz - 1) // 2].ravel())
    assert not os.path.exists("%s%d.dat" % (prefix, 10))
