"""Seeded synthetic shots for the workloads the library is measured on.

There is no field data here, so each workload is a generated earth model with
the sizes, spacings and parameter ranges of the published configurations.
Inputs are built exactly as the reference's main program builds them
(3dPureqPModeling1.0.c:234-268): interior model -> extend_model into the PML
shell -> vpmax = (1 + 2 max eps) max vp -> pmlcoff -> Source at the window
centre on the top of the interior, receivers on that plane.

The host utilities (extend_model, pmlcoff, Source, FD tables) come from the
library by default.  set_backend("oracle") takes them from the CPU oracle
instead and returns oracle problems: the CPU reference measurement builds its
inputs that way, so that its process never loads the library it is compared
with.  Both restate the same reference functions and give identical inputs.
"""
import numpy as np

_BACKEND = "qp3d"


def set_backend(name):
    """'qp3d' (default) or 'oracle' (see the module docstring)."""
    global _BACKEND
    if name not in ("qp3d", "oracle"):
        raise ValueError("unknown backend %r" % (name,))
    _BACKEND = name


class _OracleHost:
    """The oracle's restatements under the library's names."""

    def __init__(self):
        from oracle import oracle as O
        self.extend_model = O.extend_model
        self.pmlcoff = O.pmlcoff
        self.source = O.source
        self.fdcoff = O.fdcoff
        self.pml_state_size = O.pml_state_size
        self.Shot = O.Problem

    @staticmethod
    def absmax(a):
        # CPU_function.c:10-22 starts at 0 and keeps the largest |a|
        a = np.asarray(a, np.float32)
        return float(np.max(np.abs(a))) if a.size else 0.0


def _host():
    if _BACKEND == "oracle":
        return _OracleHost()
    import qp3d
    return qp3d


def _finish(vp_i, eps_i, del_i, pml, dx, dt, nt, fm, src_xyz=None, sz=None, amp=1.0,
            alpha=1.0):
    h = _host()
    nz0, hx, hy = vp_i.shape
    nx, ny, nz = hx + 2 * pml, hy + 2 * pml, nz0 + 2 * pml
    vp = h.extend_model(vp_i, nx, ny, nz, pml)
    eps = h.extend_model(eps_i, nx, ny, nz, pml)
    dl = h.extend_model(del_i, nx, ny, nz, pml)
    # float arithmetic throughout, as 3dPureqPModeling.c:227 computes vpmax
    vpmax = (np.float32(1) + np.float32(2) * np.float32(h.absmax(eps))) * \
        np.float32(h.absmax(vp))
    prof = h.pmlcoff(pml, float(vpmax), dx, dx, dx)
    if src_xyz is None:   # 3dPureqPModeling1.0.c:263-265
        src_xyz = ((hx - 1) // 2, (hy - 1) // 2, 0)
    sx, sy, sz0 = (v + pml for v in src_xyz)
    src, wav = h.source(sx, sy, sz0, fm, amp, alpha, dt, dx, dx, dx, 1.0 / fm, nt,
                        nx, ny, nz)
    c, c2 = h.fdcoff()
    if sz is None:
        sz = sz0
    return h.Shot(nx, ny, nz, pml, sz, dx, dx, dx, dt, vp, eps, dl, src, wav, prof, c, c2)


def linear_vti(h=100, nz0=100, pml=20, nt=1000, dx=10.0, dt=5e-4, fm=25.0, src=(50, 50, 5),
               vp_top=2000.0, vp_bottom=3500.0, eps=0.2, delta=0.1):
    """Plain single-shot workload: vp linear in depth, uniform eps/delta,
    point source at `src` (interior cells), receivers on the source plane.
    Defaults: 100^3 interior, 20-cell PML, 1000 steps of 0.5 ms, 25 Hz."""
    z = np.arange(nz0, dtype=np.float64)
    vpz = (vp_top + (vp_bottom - vp_top) * z / max(nz0 - 1, 1)).astype(np.float32)
    vp_i = np.broadcast_to(vpz[:, None, None], (nz0, h, h)).astype(np.float32)
    eps_i = np.full((nz0, h, h), eps, np.float32)
    del_i = np.full((nz0, h, h), delta, np.float32)
    return _finish(vp_i, eps_i, del_i, pml, dx, dt, nt, fm, src_xyz=src)


def layered_volume(hx, hy, nz0, nlayers=12, seed=2, slope=0.15):
    """Interior vp, eps, delta ([nz0][hx][hy]) of a layered model with dipping
    planar interfaces: per layer vp U[1500,4500], eps U[0,0.3],
    delta U[0,min(eps,0.15)]."""
    rng = np.random.default_rng(seed)
    z0 = np.sort(rng.uniform(0, nz0, nlayers - 1))
    ax = rng.uniform(-slope, slope, nlayers - 1)
    ay = rng.uniform(-slope, slope, nlayers - 1)
    lvp = rng.uniform(1500, 4500, nlayers).astype(np.float32)
    leps = rng.uniform(0, 0.3, nlayers).astype(np.float32)
    ldel = np.array([rng.uniform(0, min(e, 0.15)) for e in leps], np.float32)
    xs = np.arange(hx, dtype=np.float64)[:, None] - hx / 2
    ys = np.arange(hy, dtype=np.float64)[None, :] - hy / 2
    idx = np.zeros((nz0, hx, hy), np.int8)
    zz = np.arange(nz0, dtype=np.float64)[:, None, None]
    for i in range(nlayers - 1):
        depth = z0[i] + ax[i] * xs + ay[i] * ys
        idx += (zz >= depth[None]).astype(np.int8)
    return lvp[idx], leps[idx], ldel[idx]


def layered_vti(hx=400, hy=400, nz0=300, pml=30, nt=3000, dx=10.0, dt=5e-4, fm=20.0,
                nlayers=12, seed=2, slope=0.15, src=None):
    """Layered model (layered_volume).  Defaults: 400x400x300 interior,
    30-cell PML, 3000 steps, 20 Hz source at the surface centre."""
    vp_i, eps_i, del_i = layered_volume(hx, hy, nz0, nlayers, seed, slope)
    return _finish(vp_i, eps_i, del_i, pml, dx, dt, nt, fm, src_xyz=src)


def anomalous_volume(hx=800, hy=800, nz0=400, nlayers=20, nanom=30, seed=5, slope=0.15,
                     sigma=(10.0, 40.0), amp=0.15):
    """Interior vp, eps, delta of the large workload: layered_volume with
    nlayers layers plus nanom Gaussian velocity anomalies (relative amplitude
    uniform in [-amp, amp], sigma uniform in the given range of cells, centres
    uniform in the volume), each evaluated within 3 sigma of its centre."""
    vp, eps, de = layered_volume(hx, hy, nz0, nlayers, seed, slope)
    rng = np.random.default_rng(seed + 2000)
    scale = np.ones((nz0, hx, hy), np.float32)
    for _ in range(nanom):
        cz, cx, cy = rng.uniform(0, nz0), rng.uniform(0, hx), rng.uniform(0, hy)
        s = rng.uniform(*sigma)
        a = rng.uniform(-amp, amp)
        lo = [max(0, int(c - 3 * s)) for c in (cz, cx, cy)]
        hi = [min(n, int(c + 3 * s) + 1) for c, n in zip((cz, cx, cy), (nz0, hx, hy))]
        if any(h <= l for l, h in zip(lo, hi)):
            continue
        z = (np.arange(lo[0], hi[0]) - cz)[:, None, None]
        x = (np.arange(lo[1], hi[1]) - cx)[None, :, None]
        y = (np.arange(lo[2], hi[2]) - cy)[None, None, :]
        g = np.exp(-(z * z + x * x + y * y) / (2.0 * s * s)).astype(np.float32)
        scale[lo[0]:hi[0], lo[1]:hi[1], lo[2]:hi[2]] += np.float32(a) * g
    return (vp * scale).astype(np.float32), eps, de


def large_vti(hx=800, hy=800, nz0=400, pml=40, nt=5000, dx=10.0, dt=5e-4, fm=20.0, seed=5,
              decimate=1):
    """Large workload: anomalous_volume, 40-cell PML, 5000 steps.  decimate=k
    keeps every k-th cell of the full-size model (spacing k*dx) for the
    oracle comparisons."""
    vp, eps, de = anomalous_volume(hx, hy, nz0, seed=seed)
    if decimate > 1:
        k = decimate
        vp, eps, de = (np.ascontiguousarray(a[::k, ::k, ::k]) for a in (vp, eps, de))
    return _finish(vp, eps, de, pml, dx * decimate, dt, nt, fm)


def adjoint_case(hx=200, hy=200, nz0=150, pml=20, nt=2000, dx=10.0, dt=5e-4, fm=20.0, seed=4,
                 sigma=5.0, grid=4):
    """Gradient workload: a true layered model (layered_volume) and a start
    model smoothed by a 3D Gaussian of sigma cells, with grid x grid shots on
    the surface (sources at the centres of a regular grid of the top face,
    receivers on that face).  Returns (true_shots, start_shots)."""
    from scipy.ndimage import gaussian_filter
    vp, eps, de = layered_volume(hx, hy, nz0, 12, seed, 0.15)
    smooth = [gaussian_filter(a.astype(np.float64), sigma, mode="nearest").astype(np.float32)
              for a in (vp, eps, de)]
    pos = [int((i + 0.5) * hx / grid) for i in range(grid)]
    posy = [int((i + 0.5) * hy / grid) for i in range(grid)]
    true, start = [], []
    for sx in pos:
        for sy in posy:
            true.append(_finish(vp, eps, de, pml, dx, dt, nt, fm, src_xyz=(sx, sy, 0)))
            start.append(_finish(*smooth, pml, dx, dt, nt, fm, src_xyz=(sx, sy, 0)))
    return true, start


def batch_windows(nshots=64, seed=3, model=(512, 512, 200), hrange=(128, 256),
                  zrange=(128, 200), frange=(15.0, 30.0)):
    """Apertures of the batched workload: per shot (x0, y0, hx, hy, nz0, fm)
    with hx, hy uniform in hrange, nz0 in zrange (inclusive), the window
    origin uniform inside the model and the top of the window at the
    surface."""
    rng = np.random.default_rng(seed + 1000)
    mx, my, mz = model
    out = []
    for _ in range(nshots):
        hx = int(rng.integers(hrange[0], hrange[1] + 1))
        hy = int(rng.integers(hrange[0], hrange[1] + 1))
        nz0 = int(rng.integers(zrange[0], min(zrange[1], mz) + 1))
        x0 = int(rng.integers(0, mx - hx + 1))
        y0 = int(rng.integers(0, my - hy + 1))
        fm = float(rng.uniform(*frange))
        out.append((x0, y0, hx, hy, nz0, fm))
    return out


def batch_shots(nshots=64, seed=3, model=(512, 512, 200), pml=20, nt=2000, dx=10.0, dt=5e-4,
                hrange=(128, 256), zrange=(128, 200), frange=(15.0, 30.0)):
    """Batched workload: nshots windows (batch_windows) cut from one layered
    model of the given interior size (layered_volume, 12 layers), each
    extended by a pml-cell shell, with its Ricker source at the window's
    surface centre and receivers on that plane."""
    mx, my, mz = model
    vp_m, eps_m, del_m = layered_volume(mx, my, mz, 12, seed, 0.15)
    shots = []
    for x0, y0, hx, hy, nz0, fm in batch_windows(nshots, seed, model, hrange, zrange, frange):
        cut = lambda a: np.ascontiguousarray(a[:nz0, x0:x0 + hx, y0:y0 + hy])
        shots.append(_finish(cut(vp_m), cut(eps_m), cut(del_m), pml, dx, dt, nt, fm))
    return shots


def small_case(hx=22, hy=26, nz0=18, pml=8, nt=60, seed=7, fm=30.0, src=None, dt=5e-4):
    """Small non-cubic layered case for fast parity tests (every PML face and
    corner is reached within a few tens of steps)."""
    if src is None:
        src = (hx // 2, hy // 3, nz0 // 3)
    return layered_vti(hx=hx, hy=hy, nz0=nz0, pml=pml, nt=nt, dt=dt, fm=fm, nlayers=4,
                       seed=seed, slope=0.3, src=src)


def random_state(shot, seed=0, amp=1e-3):
    """Random u(k-1), u(k) and PML state (reference face layout), non-zero on
    every cell the reference updates, for single-step operator tests."""
    rng = np.random.default_rng(seed)
    nx, ny, nz, pml = shot.nx, shot.ny, shot.nz, shot.pml
    def vol():
        v = np.zeros((nz, nx, ny), np.float32)
        # smooth-ish random field so that gradients straddle the threshold
        v[5:-5, 5:-5, 5:-5] = (amp * rng.standard_normal((nz - 10, nx - 10, ny - 10))).astype(
            np.float32)
        return v.ravel()
    u_prev, u_cur = vol(), vol()
    n = _host().pml_state_size(nx, ny, nz, pml)
    pml_state = (amp * rng.standard_normal(n + 1)).astype(np.float32)
    return u_prev, u_cur, pml_state
