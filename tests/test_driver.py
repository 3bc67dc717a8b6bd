"""The modeling program around qp3d_forward (parameter file, shot loop,
muting, output files).  Parsing is checked on the CPU; the whole job on the
GPU, bit for bit against the oracle mirror built the way the reference's main
program builds each shot (3dPureqPModeling1.0.c:225-312)."""
import os

import numpy as np
import pytest

import qp3d
from oracle import oracle as O
from driver_case import CASE, oracle_direct, oracle_shot, write_case
from helpers import bits_equal


def test_parse_parameter_file(tmp_path):
    path, c, _ = write_case(str(tmp_path))
    rc, p, msg = qp3d.parse_parameter_file(path)
    assert rc == 0, msg
    assert (p.nt, p.ntsnap, p.Nx0, p.Ny0, p.Nz0) == (c["nt"], c["ntsnap"], c["Nx0"], c["Ny0"], c["Nz0"])
    assert np.float32(p.dt) == np.float32(c["dt"]) and p.dx == c["dx"] and p.fm == c["fm"]
    assert (p.sx0, p.sy0, p.nxshot, p.nyshot, p.dxshot, p.dyshot) == (12, 11, 1, 2, 6, 9)
    assert (p.hx, p.hy, p.pml, p.multishot, p.muteflag, p.snapflag_full, p.snapflag_direct) == \
        (20, 18, 8, 1, 1, 1, 0)
    assert p.vp_file.decode().endswith("/vp.dat")
    assert p.recmut_file.decode().endswith("/Record_mute.dat")
    assert p.snap_full.decode().endswith("/snapshot_fullwave")


def test_parse_errors(tmp_path):
    rc, _, msg = qp3d.parse_parameter_file(tmp_path / "missing.txt")
    assert rc == -6 and "cannot open" in msg
    path, _, _ = write_case(str(tmp_path))
    text = open(path).read().splitlines()
    text[3] = "40 36"                      # Nz0 missing: the next header is read as a value
    open(path, "w").write("\n".join(text) + "\n")
    rc, _, msg = qp3d.parse_parameter_file(path)
    assert rc == -1 and "section" in msg
    path, _, _ = write_case(str(tmp_path), hx=60)   # window wider than the model
    rc, _, msg = qp3d.parse_parameter_file(path)
    assert rc == -1


def test_rsf_header_writer(tmp_path):
    # host-only: the header text of qp3d_write_rsf_header
    f = str(tmp_path / "Record_fullwave.dat")
    assert qp3d.write_rsf_header(f, [(18, 10.0, "y"), (20, 12.5, "x"), (300, 5e-4, "t"),
                                     (4, 1.0, "shot")]) == 0
    h = qp3d.read_rsf_header(str(tmp_path / "Record_fullwave.rsf"))
    assert h["in"] == f and h["data_format"] == "native_float" and h["esize"] == "4"
    assert [h["n%d" % a] for a in range(1, 5)] == ["18", "20", "300", "4"]
    assert float(h["d2"]) == 12.5 and float(h["d3"]) == np.float32(5e-4) and h["o1"] == "0"
    assert [h["label%d" % a] for a in range(1, 5)] == ["y", "x", "t", "shot"]
    g = str(tmp_path / "snap_xz")           # no .dat suffix: .rsf appended
    assert qp3d.write_rsf_header(g, [(7, 1.0, "x")]) == 0
    assert qp3d.read_rsf_header(g + ".rsf")["n1"] == "7"
    assert qp3d.write_rsf_header(f, [(0, 1.0, "y")]) == -1        # empty axis
    assert qp3d.write_rsf_header(str(tmp_path / "no" / "x.dat"), [(1, 1.0, "y")]) == -6


def _check_rsf(d, c, nshots, snapfull):
    nt, hx, hy, Nz0 = c["nt"], c["hx"], c["hy"], c["Nz0"]
    for name in ("Record_fullwave", "Record_mute"):
        h = qp3d.read_rsf_header(os.path.join(d, name + ".rsf"))
        assert [int(h["n%d" % a]) for a in range(1, 5)] == [hy, hx, nt, nshots]
        assert h["in"].endswith(name + ".dat") and h["label3"] == "t"
    h = qp3d.read_rsf_header(os.path.join(d, "Record_direct.rsf"))
    assert [int(h["n%d" % a]) for a in range(1, 4)] == [hy, hx, nt]
    h = qp3d.read_rsf_header(os.path.join(d, "recordxz.rsf"))
    assert (int(h["n1"]), int(h["n2"])) == (hx, nt)
    if snapfull:
        h = qp3d.read_rsf_header(os.path.join(d, "snapshot_fullwave20.rsf"))
        assert [int(h["n%d" % a]) for a in range(1, 4)] == [hy, hx, Nz0]
        h = qp3d.read_rsf_header(os.path.join(d, "snapshot_fullwave_yz20.rsf"))
        assert (int(h["n1"]), int(h["n2"]), h["label2"]) == (hy, Nz0, "z")


@pytest.mark.gpu
@pytest.mark.parametrize("direct,snapfull,per_call,nxshot,rsf", [
    ("values", 1, 0, 1, 1),  # full-wave snapshots: one qp3d_forward per shot
    ("source", 1, 0, 1, 0),
    ("values", 0, 0, 2, 1),  # no snapshots: all four shots in one qp3d_batch call
    ("values", 0, 3, 2, 0),  # groups of three and one
    ("values", 0, 1, 2, 0),  # one shot per call, as the reference
])
def test_modeling_job_matches_oracle(tmp_path, direct, snapfull, per_call, nxshot, rsf):
    d = str(tmp_path)
    path, c, models = write_case(d, snapfull=snapfull, nxshot=nxshot)
    if direct == "values":
        rc, msg = qp3d.run_parameter_file(path, direct_model=qp3d.DIRECT_VALUES,
                                          direct=(2100.0, 0.1, 0.05), shots_per_call=per_call,
                                          write_rsf=rsf)
        dvals = (2100.0, 0.1, 0.05)
    else:
        rc, msg = qp3d.run_parameter_file(path, shots_per_call=per_call, write_rsf=rsf)
        fny, fnx = c["sy0"] - (c["hy"] - 1) // 2, c["sx0"] - (c["hx"] - 1) // 2
        cell = (fny + (c["hy"] - 1) // 2, fnx + (c["hx"] - 1) // 2, 0)
        dvals = tuple(float(m[cell]) for m in models)
    assert rc == 0, msg
    nt, hx, hy = c["nt"], c["hx"], c["hy"]
    rec_dir, _, _ = O.run(O.MIRROR, oracle_direct(O, c, dvals))
    got_dir = np.fromfile(os.path.join(d, "Record_direct.dat"), np.float32)
    assert bits_equal(got_dir, rec_dir.ravel())
    full = np.fromfile(os.path.join(d, "Record_fullwave.dat"), np.float32).reshape(-1, nt, hx, hy)
    mute = np.fromfile(os.path.join(d, "Record_mute.dat"), np.float32).reshape(-1, nt, hx, hy)
    shots = [(c["sx0"] + ix * c["dxshot"], c["sy0"] + iy * c["dyshot"])
             for ix in range(c["nxshot"]) for iy in range(c["nyshot"])]
    assert full.shape[0] == len(shots) and mute.shape[0] == len(shots)   # appended shot by shot
    if rsf:
        _check_rsf(d, c, len(shots), snapfull)
    else:
        assert not os.path.exists(os.path.join(d, "Record_fullwave.rsf"))
    last = None
    for i, (sx, sy) in enumerate(shots):
        prob = oracle_shot(O, c, models, sx, sy)
        rec, _, _ = O.run(O.MIRROR, prob)
        assert bits_equal(full[i], rec), "shot %d" % i
        assert bits_equal(mute[i], (rec - rec_dir).astype(np.float32))
        last = prob
        if i == 0:
            xz = np.fromfile(os.path.join(d, "recordxz.dat"), np.float32).reshape(nt, hx)
            yz = np.fromfile(os.path.join(d, "recordyz.dat"), np.float32).reshape(nt, hy)
            assert bits_equal(xz, rec[:, :, (hy - 1) // 2])
            assert bits_equal(yz, rec[:, (hx - 1) // 2, :])
    if not snapfull:
        assert not os.path.exists(os.path.join(d, "snapshot_fullwave0.dat"))
        return
    # snapshots of the last shot (each shot overwrites the same names)
    pml, Nz0 = c["pml"], c["Nz0"]
    st = None
    done = 0
    for k in (0, 20):
        _, _, st = O.run(O.MIRROR, last, k0=done, nsteps=k + 1 - done, state=st, want_record=False)
        done = k + 1
        u = st.u2.reshape(last.nz, last.nx, last.ny)[pml:pml + Nz0, pml:pml + hx, pml:pml + hy]
        snap = np.fromfile(os.path.join(d, "snapshot_fullwave%d.dat" % k), np.float32)
        assert bits_equal(snap, u.ravel())
        sxz = np.fromfile(os.path.join(d, "snapshot_fullwave_xz%d.dat" % k), np.float32)
        assert bits_equal(sxz, u[:, :, (hy - 1) // 2].ravel())


def test_modeling_program_without_device_fails_cleanly(tmp_path):
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    path, _, _ = write_case(str(tmp_path))
    rc, msg = qp3d.run_parameter_file(path)
    assert rc == -2 and "device" in msg
