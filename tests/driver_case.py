"""A small modeling job in the reference's parameter-file format, and the
oracle's view of what it must produce (shared by the driver tests)."""
import os

import numpy as np

PARAM_TEMPLATE = """Time sampling rate[dt-s]--record time length[nt]--snapshot interval
{dt}\t{nt}\t\t{ntsnap}
X-direction distance--y-direction distance--z-direction distance (cells)
{Nx0}\t  {Ny0}     {Nz0}
X-direction sampling internal--y-direction--z-direction[m]
{dx}\t{dx}   \t{dx}
Ricker wavelet dominant frequency--source amplitude--source decay coefficient[alp]
{fm}\t{amp}    \t{alpha}
First source position x y z (cells)
{sx0}\t\t{sy0}     \t0
First geophone position x y z
0  \t\t0  \t\t0
Nshot(x,y)--shot_interval(x,y)
{nxshot}  \t\t{nyshot}  \t\t{dxshot}  \t{dyshot}
Offset-the aperture in x and y (cells)
{hx}  \t{hy}
The number of PML absorbing boundary layers[npml]
{pml}
Model-parameters-vp-epsilon-delta-filename
{d}/vp.dat\t{d}/epsilon.dat\t{d}/delta.dat
Record-fullwave-directwave-mute-filename
{d}/Record_fullwave.dat   \t{d}/Record_direct.dat   {d}/Record_mute.dat
Record-fullwave-xoz and yoz-slice
{d}/recordxz.dat   \t{d}/recordyz.dat
Snapshot-fullwave-directwave-filename
{d}/snapshot_direct  \t{d}/snapshot_fullwave
Single-shot or multi-shots (single = 0, multi = 1)
1
Mute directwave or not(yes = 1, no = 0)
{mute}
Save fullwave wavefield snapshot or not(yes = 1, no = 0)
{snapfull}
Save directwave wavefield snapshot or not(yes = 1, no = 0)
0
"""

CASE = dict(dt=5e-4, nt=40, ntsnap=20, Nx0=40, Ny0=36, Nz0=16, dx=10.0, fm=30.0, amp=1.0,
            alpha=1.0, sx0=12, sy0=11, nxshot=1, nyshot=2, dxshot=6, dyshot=9, hx=20, hy=18,
            pml=8, mute=1, snapfull=1)


def write_case(d, **over):
    """Model files (stored [Ny0][Nx0][Nz0], z fastest) and parameter.txt."""
    c = dict(CASE, **over)
    rng = np.random.default_rng(42)
    Nx0, Ny0, Nz0 = c["Nx0"], c["Ny0"], c["Nz0"]
    z = np.arange(Nz0)[None, None, :]
    x = np.arange(Nx0)[None, :, None]
    vp = (2000.0 + 60.0 * z + 5.0 * x + 10.0 * rng.standard_normal((Ny0, Nx0, Nz0))).astype(np.float32)
    eps = np.clip(0.1 + 0.01 * rng.standard_normal((Ny0, Nx0, Nz0)), 0, 0.3).astype(np.float32)
    de = (0.5 * eps).astype(np.float32)
    for name, a in (("vp.dat", vp), ("epsilon.dat", eps), ("delta.dat", de)):
        a.tofile(os.path.join(d, name))
    path = os.path.join(d, "parameter.txt")
    with open(path, "w") as f:
        f.write(PARAM_TEMPLATE.format(d=d, **c))
    return path, c, (vp, eps, de)


def oracle_shot(O, c, models, sx, sy):
    """The oracle Problem of one shot, built as the reference's main builds it."""
    hx, hy, Nz0, pml = c["hx"], c["hy"], c["Nz0"], c["pml"]
    nx, ny, nz = hx + 2 * pml, hy + 2 * pml, Nz0 + 2 * pml
    fny, fnx = sy - (hy - 1) // 2, sx - (hx - 1) // 2
    vols = []
    for m in models:
        win = m[fny:fny + hy, fnx:fnx + hx, :].transpose(2, 1, 0)   # -> [z][x][y]
        vols.append(O.extend_model(np.ascontiguousarray(win), nx, ny, nz, pml))
    return _finish(O, c, vols)


def oracle_direct(O, c, values):
    hx, hy, Nz0, pml = c["hx"], c["hy"], c["Nz0"], c["pml"]
    n = (hx + 2 * pml) * (hy + 2 * pml) * (Nz0 + 2 * pml)
    return _finish(O, c, [np.full(n, v, np.float32) for v in values])


def _finish(O, c, vols):
    hx, hy, Nz0, pml = c["hx"], c["hy"], c["Nz0"], c["pml"]
    nx, ny, nz = hx + 2 * pml, hy + 2 * pml, Nz0 + 2 * pml
    vp, eps, de = vols
    # float arithmetic throughout, as 3dPureqPModeling1.0.c computes vpmax
    e = np.float32(O.lib().oracle_absmax(O._ptr(eps), eps.size))
    v = np.float32(O.lib().oracle_absmax(O._ptr(vp), vp.size))
    vpmax = (np.float32(1) + np.float32(2) * e) * v
    prof = O.pmlcoff(pml, float(vpmax), c["dx"], c["dx"], c["dx"])
    sx1, sy1, sz1 = (hx - 1) // 2 + pml, (hy - 1) // 2 + pml, pml
    src, wav = O.source(sx1, sy1, sz1, c["fm"], c["amp"], c["alpha"], c["dt"], c["dx"], c["dx"],
                        c["dx"], np.float32(1.0 / c["fm"]), c["nt"], nx, ny, nz)
    cc, cc2 = O.fdcoff()
    return O.Problem(nx, ny, nz, pml, pml, c["dx"], c["dx"], c["dx"], c["dt"], vp, eps, de, src,
                     wav, prof, cc, cc2)
