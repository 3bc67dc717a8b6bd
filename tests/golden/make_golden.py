"""Generate the golden vectors in this directory from the reference itself.

Runs the reference's own CPU operators (CPU_function.c compiled from the
reference checkout by oracle/build.py, driven by oracle/ref_harness.cpp) on
small seeded shots and stores inputs and outputs as .npz:

  inputs : geometry, vp, epsilon, delta, source, wavelet, damping profiles,
           FD tables (as the reference's Source/pmlcoff/fdcoff1/2 make them)
  outputs: record [nt][hx][hy], uxyzMax per step, final u(k-1), u(k) and PML
           state (reference face layout)

The reference's shipped output/*.dat files cannot serve as golden vectors
(their model files are not in the repository), so these are generated.
Usage:  python tests/golden/make_golden.py
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402

# name: (hx, hy, nz0, pml, nt, src (interior), sz (interior z), seed, fm, alpha)
CASES = {
    "layered_small": (22, 26, 18, 8, 80, (11, 8, 6), 6, 7, 30.0, 1.0),
    "pml5_wide_source": (16, 20, 14, 5, 50, (7, 9, 4), 2, 11, 35.0, 0.08),
}


def make_inputs(hx, hy, nz0, pml, nt, src, sz_i, seed, fm, alpha):
    """Seeded layered model built with the reference's own host utilities."""
    rl = O.ref_lib()
    rng = np.random.default_rng(seed)
    nx, ny, nz = hx + 2 * pml, hy + 2 * pml, nz0 + 2 * pml
    # four depth bands with a checkerboard step of one band (dipping-ish edges)
    lay = np.broadcast_to((np.arange(nz0) * 4 // nz0)[:, None, None], (nz0, hx, hy))
    tilt = (np.arange(hx)[None, :, None] // 7 + np.arange(hy)[None, None, :] // 9) % 2
    lay = np.clip(lay + tilt, 0, 4)
    lvp = rng.uniform(1500, 4500, 5).astype(np.float32)
    leps = rng.uniform(0, 0.3, 5).astype(np.float32)
    ldel = np.array([rng.uniform(0, min(e, 0.15)) for e in leps], np.float32)
    vp_i, eps_i, del_i = lvp[lay], leps[lay], ldel[lay]
    vols = []
    for v in (vp_i, eps_i, del_i):
        out = np.zeros(nx * ny * nz, np.float32)
        inp = np.ascontiguousarray(v, np.float32).ravel()
        rl.ref_extend_model(O._ptr(inp), O._ptr(out), nx, ny, nz, pml)
        vols.append(out)
    vp, eps, dl = vols
    # float arithmetic throughout, as 3dPureqPModeling.c:227 computes vpmax
    vpmax = (np.float32(1) + np.float32(2) * np.float32(rl.ref_absmax(O._ptr(eps), nx, ny, nz))) \
        * np.float32(rl.ref_absmax(O._ptr(vp), nx, ny, nz))
    prof = [np.zeros(pml, np.float32) for _ in range(6)]
    dx = 10.0
    dt = 5e-4
    rl.ref_pmlcoff(pml, vpmax, dx, dx, dx, *[O._ptr(p) for p in prof])
    source = np.zeros(nx * ny * nz, np.float32)
    wavelet = np.zeros(nt, np.float32)
    rl.ref_source(src[0] + pml, src[1] + pml, src[2] + pml, fm, 1.0, alpha, dt, dx, dx, dx,
                  1.0 / fm, nt, nx, ny, nz, O._ptr(source), O._ptr(wavelet))
    c = np.zeros(36, np.float32)
    c2 = np.zeros(36, np.float32)
    rl.ref_fdcoff(O._ptr(c), O._ptr(c2))
    return O.Problem(nx, ny, nz, pml, sz_i + pml, dx, dx, dx, dt, vp, eps, dl, source,
                     wavelet, prof, c, c2), float(vpmax), (vp_i, eps_i, del_i)


def main():
    if O.ref_lib() is None:
        raise SystemExit("reference CPU operators not available (oracle/build.py)")
    for name, spec in CASES.items():
        prob, vpmax, interior = make_inputs(*spec)
        rec, mx, st = O.run_reference(prob)
        np.savez_compressed(
            os.path.join(HERE, name + ".npz"),
            geom=np.array([prob.nx, prob.ny, prob.nz, prob.pml, prob.sz], np.int32),
            spacing=np.array([prob.dx, prob.dy, prob.dz, prob.dt], np.float32),
            vpmax=np.float32(vpmax),
            vp_interior=interior[0], eps_interior=interior[1], del_interior=interior[2],
            vp=prob.vp, eps=prob.eps, delta=prob.delta, source=prob.src,
            wavelet=prob.wavelet, prof=np.stack(prob.prof), c=prob.c, c2=prob.c2,
            record=rec, uxyzmax=mx, u_prev=st.u1, u_cur=st.u2, pml_state=st.pml)
        print(name, "nt=%d" % prob.nt, "peak=%.3e" % np.abs(rec).max(),
              "nnz(source)=%d" % np.count_nonzero(prob.src))


if __name__ == "__main__":
    main()
