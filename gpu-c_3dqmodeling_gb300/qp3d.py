"""ctypes bindings of libqp3d.so (the C ABI in include/qp3d.h).

The library is the product; this module only marshals numpy arrays.  It never
falls back to any other implementation: if the shared library is missing or a
CUDA device is unavailable, calls raise.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "lib", "libqp3d.so")

QP3D_OK = 0
ERRORS = {-1: "invalid argument", -2: "CUDA error", -3: "out of memory",
          -4: "device wait timed out", -5: "invalid call order", -6: "file I/O error",
          -7: "snapshot callback failed"}
SNAP_VOLUME, SNAP_XZ, SNAP_YZ, SNAP_XY = 0, 1, 2, 3

_f32p = ctypes.POINTER(ctypes.c_float)
_vp = ctypes.c_void_p


class Geom(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("nt", ctypes.c_int), ("pml", ctypes.c_int), ("sz", ctypes.c_int),
                ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                ("dt", ctypes.c_float)]


class Model(ctypes.Structure):
    _fields_ = [(n, _f32p) for n in ("vp", "epsilon", "delta", "source", "wavelet", "dlr",
                                      "ddlr", "dtb", "ddtb", "dfb", "ddfb", "c", "c2")]


class ShotDesc(ctypes.Structure):
    """qp3d_shot: one shot of qp3d_batch."""
    _fields_ = [("geom", Geom), ("model", Model), ("record", _f32p)]


class BatchStats(ctypes.Structure):
    _fields_ = [("groups", ctypes.c_int), ("batched_shots", ctypes.c_int),
                ("single_shots", ctypes.c_int), ("candidate", ctypes.c_int),
                ("tile_rows", ctypes.c_int), ("zblocks", ctypes.c_int), ("tuned", ctypes.c_int),
                ("ncand", ctypes.c_int), ("cand_ms", ctypes.c_float * 8),
                ("graph_steps", ctypes.c_int), ("redo_steps", ctypes.c_int),
                ("work_items", ctypes.c_int), ("ctas", ctypes.c_int), ("run_ms", ctypes.c_float)]

    def as_dict(self):
        d = {n: getattr(self, n) for n, _ in self._fields_ if n != "cand_ms"}
        d["cand_ms"] = [round(float(v), 4) for v in self.cand_ms[:self.ncand]]
        return d


SNAP_FN = ctypes.CFUNCTYPE(ctypes.c_int, ctypes.c_void_p, ctypes.c_int, ctypes.c_int,
                           _f32p, ctypes.c_int, ctypes.c_int, ctypes.c_int)


class Snap(ctypes.Structure):
    _fields_ = [("ntsnap", ctypes.c_int), ("kinds", ctypes.c_uint), ("fn", SNAP_FN),
                ("user", ctypes.c_void_p)]


PATH_MAX = 256


class Parameters(ctypes.Structure):
    _fields_ = ([("dt", ctypes.c_float), ("nt", ctypes.c_int), ("ntsnap", ctypes.c_int),
                 ("Nx0", ctypes.c_int), ("Ny0", ctypes.c_int), ("Nz0", ctypes.c_int),
                 ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
                 ("fm", ctypes.c_float), ("amp", ctypes.c_float), ("alpha", ctypes.c_float),
                 ("sx0", ctypes.c_int), ("sy0", ctypes.c_int), ("sz0", ctypes.c_int),
                 ("gx0", ctypes.c_int), ("gy0", ctypes.c_int), ("gz0", ctypes.c_int),
                 ("nxshot", ctypes.c_int), ("nyshot", ctypes.c_int), ("dxshot", ctypes.c_int),
                 ("dyshot", ctypes.c_int), ("hx", ctypes.c_int), ("hy", ctypes.c_int),
                 ("pml", ctypes.c_int)] +
                [(n, ctypes.c_char * PATH_MAX) for n in (
                    "vp_file", "eps_file", "del_file", "recfull_file", "recdir_file",
                    "recmut_file", "recxz_file", "recyz_file", "snap_direct", "snap_full")] +
                [("multishot", ctypes.c_int), ("muteflag", ctypes.c_int),
                 ("snapflag_full", ctypes.c_int), ("snapflag_direct", ctypes.c_int)])


DIRECT_SOURCE_CELL, DIRECT_ZERO, DIRECT_VALUES = 0, 1, 2


class RunOptions(ctypes.Structure):
    _fields_ = [("device", ctypes.c_int), ("direct_model", ctypes.c_int),
                ("direct_vp", ctypes.c_float), ("direct_eps", ctypes.c_float),
                ("direct_del", ctypes.c_float), ("verbose", ctypes.c_int),
                ("shots_per_call", ctypes.c_int), ("write_rsf", ctypes.c_int)]


# every symbol include/qp3d.h and include/qp3d_driver.h declare
EXPORTS = [
    "qp3d_version", "qp3d_strerror", "qp3d_ctx_create", "qp3d_ctx_destroy",
    "qp3d_ctx_last_error", "qp3d_forward", "qp3d_adjoint", "qp3d_batch", "qp3d_batch_get_stats", "qp3d_shot_load", "qp3d_shot_reset",
    "qp3d_shot_advance", "qp3d_shot_sync", "qp3d_shot_step", "qp3d_shot_read_record",
    "qp3d_shot_read_uxyzmax", "qp3d_shot_read_stats", "qp3d_shot_snapshot", "qp3d_pml_state_size",
    "qp3d_shot_write_state", "qp3d_shot_read_state", "qp3d_shot_time",
    "qp3d_shot_launches_per_step", "qp3d_ctx_launch_count", "qp3d_tune", "qp3d_tune_get", "qp3d_event_record",
    "qp3d_event_elapsed",
    "qp3d_host_alloc", "qp3d_host_free", "qp3d_gradmax_noalloc", "qp3d_fdcoff1", "qp3d_fdcoff2", "qp3d_pmlcoff",
    "qp3d_source", "qp3d_extend_model", "qp3d_absmax", "qp3d_readmodel3d",
    "qp3d_parse_parameter_file", "qp3d_run_parameter_file", "qp3d_write_rsf_header",
]

_lib = None


def load():
    """Load libqp3d.so (built by build.py); raises if it is missing."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("libqp3d.so is not built (%s); run build.py" % LIB_PATH)
    L = ctypes.CDLL(LIB_PATH)
    P = ctypes.POINTER
    sig = {
        "qp3d_version": (ctypes.c_int, []),
        "qp3d_strerror": (ctypes.c_char_p, [ctypes.c_int]),
        "qp3d_ctx_create": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_void_p)]),
        "qp3d_ctx_destroy": (None, [_vp]),
        "qp3d_ctx_last_error": (ctypes.c_char_p, [_vp]),
        "qp3d_forward": (ctypes.c_int, [_vp, P(Geom), P(Model), _vp, P(Snap)]),
        "qp3d_batch": (ctypes.c_int, [_vp, ctypes.c_int, P(ShotDesc)]),
        "qp3d_adjoint": (ctypes.c_int, [_vp, P(Geom), P(Model), _vp, _vp, _vp, _vp, _vp]),
        "qp3d_batch_get_stats": (ctypes.c_int, [_vp, P(BatchStats)]),
        "qp3d_shot_load": (ctypes.c_int, [_vp, P(Geom), P(Model)]),
        "qp3d_shot_reset": (ctypes.c_int, [_vp]),
        "qp3d_shot_advance": (ctypes.c_int, [_vp, ctypes.c_int]),
        "qp3d_shot_sync": (ctypes.c_int, [_vp]),
        "qp3d_shot_step": (ctypes.c_int, [_vp]),
        "qp3d_shot_read_record": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp]),
        "qp3d_shot_read_uxyzmax": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp]),
        "qp3d_shot_read_stats": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
        "qp3d_shot_snapshot": (ctypes.c_int, [_vp, P(Snap)]),
        "qp3d_pml_state_size": (ctypes.c_size_t, [ctypes.c_int] * 4),
        "qp3d_shot_write_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, _vp]),
        "qp3d_shot_read_state": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
        "qp3d_shot_time": (ctypes.c_int, [_vp, ctypes.c_int, P(ctypes.c_float),
                                          P(ctypes.c_float), P(ctypes.c_float)]),
        "qp3d_shot_launches_per_step": (ctypes.c_int, [_vp]),
        "qp3d_ctx_launch_count": (ctypes.c_longlong, [_vp]),
        "qp3d_tune": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
        "qp3d_tune_get": (ctypes.c_int, [_vp, ctypes.c_char_p]),
        "qp3d_event_record": (ctypes.c_int, [_vp, ctypes.c_int]),
        "qp3d_event_elapsed": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int,
                                              P(ctypes.c_float)]),
        "qp3d_host_alloc": (ctypes.c_void_p, [ctypes.c_size_t]),
        "qp3d_host_free": (None, [_vp]),
        "qp3d_gradmax_noalloc": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                ctypes.c_int, ctypes.c_float, ctypes.c_float,
                                                ctypes.c_float, _vp, _vp, _vp, ctypes.c_char_p,
                                                ctypes.c_size_t]),
        "qp3d_fdcoff1": (None, [_vp]),
        "qp3d_fdcoff2": (None, [_vp]),
        "qp3d_pmlcoff": (None, [ctypes.c_int] + [ctypes.c_float] * 4 + [_vp] * 6),
        "qp3d_source": (None, [ctypes.c_int] * 3 + [ctypes.c_float] * 8 +
                        [ctypes.c_int] * 4 + [_vp] * 2),
        "qp3d_extend_model": (None, [_vp, _vp] + [ctypes.c_int] * 4),
        "qp3d_absmax": (ctypes.c_float, [_vp, ctypes.c_size_t]),
        "qp3d_readmodel3d": (ctypes.c_int, [ctypes.c_char_p, _vp] + [ctypes.c_int] * 9),
        "qp3d_parse_parameter_file": (ctypes.c_int, [ctypes.c_char_p, P(Parameters),
                                                     ctypes.c_char_p, ctypes.c_size_t]),
        "qp3d_run_parameter_file": (ctypes.c_int, [ctypes.c_char_p, P(RunOptions),
                                                   ctypes.c_char_p, ctypes.c_size_t]),
        "qp3d_write_rsf_header": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int,
                                                 P(ctypes.c_longlong), P(ctypes.c_float),
                                                 P(ctypes.c_char_p)]),
    }
    for name, (res, args) in sig.items():
        f = getattr(L, name)
        f.restype = res
        f.argtypes = args
    _lib = L
    return L


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _fp(a):
    return None if a is None else a.ctypes.data_as(_f32p)


class QP3DError(RuntimeError):
    pass


# ---------------------------------------------------------------------------
# host utilities
# ---------------------------------------------------------------------------
def fdcoff():
    c = np.zeros(36, np.float32)
    c2 = np.zeros(36, np.float32)
    load().qp3d_fdcoff1(_p(c))
    load().qp3d_fdcoff2(_p(c2))
    return c, c2


def pmlcoff(pml, vpmax, dx, dy, dz):
    out = [np.zeros(max(pml, 1), np.float32) for _ in range(6)]
    load().qp3d_pmlcoff(pml, vpmax, dx, dy, dz, *[_p(o) for o in out])
    return out   # dlr, ddlr, dtb, ddtb, dfb, ddfb


def source(sx, sy, sz, fm, amp, alpha, dt, dx, dy, dz, t0, nt, nx, ny, nz):
    src = np.zeros(nx * ny * nz, np.float32)
    wav = np.zeros(nt, np.float32)
    load().qp3d_source(sx, sy, sz, fm, amp, alpha, dt, dx, dy, dz, t0, nt, nx, ny, nz,
                       _p(src), _p(wav))
    return src, wav


def extend_model(interior, nx, ny, nz, pml):
    out = np.empty(nx * ny * nz, np.float32)
    inp = np.ascontiguousarray(interior, np.float32).ravel()
    load().qp3d_extend_model(_p(inp), _p(out), nx, ny, nz, pml)
    return out


def absmax(a):
    a = np.ascontiguousarray(a, np.float32).ravel()
    return float(load().qp3d_absmax(_p(a), a.size))


def parse_parameter_file(path):
    """qp3d_parse_parameter_file -> (rc, Parameters, message)."""
    prm = Parameters()
    err = ctypes.create_string_buffer(512)
    rc = load().qp3d_parse_parameter_file(str(path).encode(), ctypes.byref(prm), err, len(err))
    return rc, prm, err.value.decode()


def run_parameter_file(path, device=0, direct_model=DIRECT_SOURCE_CELL, direct=(0.0, 0.0, 0.0),
                       verbose=False, shots_per_call=0, write_rsf=False):
    """qp3d_run_parameter_file -> (rc, message)."""
    o = RunOptions(device, direct_model, direct[0], direct[1], direct[2], int(verbose),
                   int(shots_per_call), int(write_rsf))
    err = ctypes.create_string_buffer(512)
    rc = load().qp3d_run_parameter_file(str(path).encode(), ctypes.byref(o), err, len(err))
    return rc, err.value.decode()


def write_rsf_header(datafile, axes):
    """qp3d_write_rsf_header; axes = [(n, d, label), ...] fastest first -> rc."""
    k = len(axes)
    n = (ctypes.c_longlong * k)(*[int(a[0]) for a in axes])
    d = (ctypes.c_float * k)(*[float(a[1]) for a in axes])
    lab = (ctypes.c_char_p * k)(*[str(a[2]).encode() for a in axes])
    return int(load().qp3d_write_rsf_header(str(datafile).encode(), k, n, d, lab))


def read_rsf_header(path):
    """key -> value (str, quotes removed) of an RSF header file."""
    out = {}
    for line in open(path):
        line = line.strip()
        if "=" in line:
            key, v = line.split("=", 1)
            out[key] = v.strip('"')
    return out


def pml_state_size(nx, ny, nz, pml):
    return int(load().qp3d_pml_state_size(nx, ny, nz, pml))


# ---------------------------------------------------------------------------
# shot inputs
# ---------------------------------------------------------------------------
class Shot:
    """One shot's inputs in the reference layout (padded [nz][nx][ny] volumes)."""

    def __init__(self, nx, ny, nz, pml, sz, dx, dy, dz, dt, vp, eps, delta, src, wavelet,
                 prof, c, c2):
        f = lambda a: np.ascontiguousarray(a, np.float32).ravel()
        self.nx, self.ny, self.nz, self.pml, self.sz = nx, ny, nz, pml, sz
        self.dx, self.dy, self.dz, self.dt = dx, dy, dz, dt
        self.vp, self.eps, self.delta = f(vp), f(eps), f(delta)
        self.src = None if src is None else f(src)
        self.wavelet = f(wavelet)
        self.prof = [f(p) for p in prof]
        self.c, self.c2 = f(c), f(c2)

    @property
    def nt(self):
        return int(self.wavelet.size)

    @property
    def N(self):
        return self.nx * self.ny * self.nz

    @property
    def hx(self):
        return self.nx - 2 * self.pml

    @property
    def hy(self):
        return self.ny - 2 * self.pml

    def geom(self, nt=None):
        g = Geom()
        g.nx, g.ny, g.nz = self.nx, self.ny, self.nz
        g.nt = self.nt if nt is None else nt
        g.pml, g.sz = self.pml, self.sz
        g.dx, g.dy, g.dz, g.dt = self.dx, self.dy, self.dz, self.dt
        return g

    def model(self):
        m = Model()
        m.vp, m.epsilon, m.delta = _fp(self.vp), _fp(self.eps), _fp(self.delta)
        m.source, m.wavelet = _fp(self.src), _fp(self.wavelet)
        m.dlr, m.ddlr, m.dtb, m.ddtb, m.dfb, m.ddfb = [_fp(p) for p in self.prof]
        m.c, m.c2 = _fp(self.c), _fp(self.c2)
        return m

    def to_oracle(self, O):
        """The same inputs as an oracle Problem (tests only)."""
        return O.Problem(self.nx, self.ny, self.nz, self.pml, self.sz, self.dx, self.dy,
                         self.dz, self.dt, self.vp, self.eps, self.delta, self.src,
                         self.wavelet, self.prof, self.c, self.c2)


# ---------------------------------------------------------------------------
# context
# ---------------------------------------------------------------------------
class Context:
    def __init__(self, device=0):
        self._L = load()
        h = ctypes.c_void_p()
        rc = self._L.qp3d_ctx_create(device, ctypes.byref(h))
        if rc != QP3D_OK:
            raise QP3DError("qp3d_ctx_create(%d) failed: %s" % (device, ERRORS.get(rc, rc)))
        self.h = h
        self.device = device
        self._shot = None

    def close(self):
        if self.h:
            self._L.qp3d_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def _check(self, rc, what):
        if rc != QP3D_OK:
            msg = self._L.qp3d_ctx_last_error(self.h)
            raise QP3DError("%s failed (%d %s): %s" % (what, rc, ERRORS.get(rc, ""),
                                                        msg.decode() if msg else ""))

    # whole shot through the C ABI
    def forward(self, shot, snap=None, record=None):
        if record is None:
            record = np.empty((shot.nt, shot.hx, shot.hy), np.float32)
        if record.size != shot.nt * shot.hx * shot.hy or record.dtype != np.float32 or \
                not record.flags.c_contiguous:
            raise ValueError("record must be a contiguous float32 array of nt*hx*hy")
        g, m = shot.geom(), shot.model()
        sp = ctypes.byref(snap) if snap is not None else None
        self._shot = None
        self._check(self._L.qp3d_forward(self.h, ctypes.byref(g), ctypes.byref(m),
                                         _p(record), sp), "qp3d_forward")
        self._shot = shot
        return record

    def batch(self, shots, records=None):
        """Run many shots with qp3d_batch; returns their records."""
        if records is None:
            records = [np.empty((s.nt, s.hx, s.hy), np.float32) for s in shots]
        arr = (ShotDesc * max(len(shots), 1))()
        keep = []
        for i, (s, r) in enumerate(zip(shots, records)):
            if r.size != s.nt * s.hx * s.hy or r.dtype != np.float32 or not r.flags.c_contiguous:
                raise ValueError("record %d must be a contiguous float32 array of nt*hx*hy" % i)
            arr[i].geom = s.geom()
            arr[i].model = s.model()
            arr[i].record = r.ctypes.data_as(_f32p)
            keep.append(r)
        self._shot = None
        self._check(self._L.qp3d_batch(self.h, len(shots), arr), "qp3d_batch")
        return records

    def adjoint(self, shot, d_obs, grads=None):
        """qp3d_adjoint: (misfit, [g_vp, g_eps, g_delta]) with the gradients
        added to grads (three float64 arrays of shot.N) when given."""
        if grads is None:
            grads = [np.zeros(shot.N, np.float64) for _ in range(3)]
        d = np.ascontiguousarray(d_obs, np.float32)
        if d.size != shot.nt * shot.hx * shot.hy:
            raise ValueError("d_obs must hold nt*hx*hy samples")
        J = ctypes.c_double()
        g, m = shot.geom(), shot.model()
        self._shot = None
        self._check(self._L.qp3d_adjoint(self.h, ctypes.byref(g), ctypes.byref(m), _p(d),
                                          _p(grads[0]), _p(grads[1]), _p(grads[2]),
                                          ctypes.byref(J)), "qp3d_adjoint")
        self._shot = shot
        return J.value, grads

    def batch_stats(self):
        st = BatchStats()
        self._check(self._L.qp3d_batch_get_stats(self.h, ctypes.byref(st)), "qp3d_batch_get_stats")
        return st.as_dict()

    def load(self, shot, nt=None):
        g, m = shot.geom(nt), shot.model()
        self._check(self._L.qp3d_shot_load(self.h, ctypes.byref(g), ctypes.byref(m)),
                    "qp3d_shot_load")
        self._shot = shot

    def reset(self):
        self._check(self._L.qp3d_shot_reset(self.h), "qp3d_shot_reset")

    def advance(self, n):
        self._check(self._L.qp3d_shot_advance(self.h, n), "qp3d_shot_advance")

    def sync(self):
        self._check(self._L.qp3d_shot_sync(self.h), "qp3d_shot_sync")

    @property
    def step(self):
        return int(self._L.qp3d_shot_step(self.h))

    def record(self, k0=0, n=None):
        s = self._loaded()
        if n is None:
            n = self.step - k0
        out = np.empty((n, s.hx, s.hy), np.float32)
        self._check(self._L.qp3d_shot_read_record(self.h, k0, n, _p(out)), "read_record")
        return out

    def uxyzmax(self, k0=0, n=None):
        if n is None:
            n = self.step - k0
        out = np.empty(n, np.float32)
        self._check(self._L.qp3d_shot_read_uxyzmax(self.h, k0, n, _p(out)), "read_uxyzmax")
        return out

    def stats(self, k0=0, n=None):
        """(re-run flags, deferred-cell counts) per step."""
        if n is None:
            n = self.step - k0
        redo = np.zeros(n, np.int32)
        alt = np.zeros(n, np.uint32)
        self._check(self._L.qp3d_shot_read_stats(self.h, k0, n, _p(redo), _p(alt)), "read_stats")
        return redo, alt

    def write_state(self, step, u_prev=None, u_cur=None, pml=None):
        f = lambda a: None if a is None else np.ascontiguousarray(a, np.float32)
        u_prev, u_cur, pml = f(u_prev), f(u_cur), f(pml)
        self._check(self._L.qp3d_shot_write_state(self.h, step, _p(u_prev), _p(u_cur), _p(pml)),
                    "write_state")

    def _loaded(self):
        if self._shot is None:
            raise QP3DError("no shot loaded through this binding")
        return self._shot

    def read_state(self):
        s = self._loaded()
        u_prev = np.empty(s.N, np.float32)
        u_cur = np.empty(s.N, np.float32)
        pml = np.empty(pml_state_size(s.nx, s.ny, s.nz, s.pml) + 1, np.float32)
        self._check(self._L.qp3d_shot_read_state(self.h, _p(u_prev), _p(u_cur), _p(pml)),
                    "read_state")
        return u_prev, u_cur, pml

    def time(self, n, per_kernel=True):
        t = ctypes.c_float()
        ts = ctypes.c_float()
        tg = ctypes.c_float()
        if per_kernel:
            rc = self._L.qp3d_shot_time(self.h, n, ctypes.byref(t), ctypes.byref(ts),
                                        ctypes.byref(tg))
        else:
            rc = self._L.qp3d_shot_time(self.h, n, ctypes.byref(t), None, None)
        self._check(rc, "qp3d_shot_time")
        return t.value, (ts.value if per_kernel else None), (tg.value if per_kernel else None)

    def launches_per_step(self):
        return int(self._L.qp3d_shot_launches_per_step(self.h))

    def launch_count(self):
        return int(self._L.qp3d_ctx_launch_count(self.h))

    def tune(self, **kv):
        for key, value in kv.items():
            self._check(self._L.qp3d_tune(self.h, key.encode(), int(value)), "qp3d_tune " + key)

    def tuning(self, key):
        return int(self._L.qp3d_tune_get(self.h, key.encode()))

    def event(self, slot):
        self._check(self._L.qp3d_event_record(self.h, slot), "qp3d_event_record")

    def elapsed(self, a, b):
        ms = ctypes.c_float()
        self._check(self._L.qp3d_event_elapsed(self.h, a, b, ctypes.byref(ms)), "event_elapsed")
        return ms.value

    def snapshot(self, snap):
        self._check(self._L.qp3d_shot_snapshot(self.h, ctypes.byref(snap)), "qp3d_shot_snapshot")


class PinnedArray:
    """A numpy view of page-locked host memory from qp3d_host_alloc."""

    def __init__(self, shape, dtype=np.float32):
        self._L = load()
        n = int(np.prod(shape)) * np.dtype(dtype).itemsize
        self.ptr = self._L.qp3d_host_alloc(max(n, 1))
        if not self.ptr:
            raise QP3DError("qp3d_host_alloc(%d) failed" % n)
        buf = (ctypes.c_char * max(n, 1)).from_address(self.ptr)
        self.array = np.frombuffer(buf, dtype=dtype, count=int(np.prod(shape))).reshape(shape)

    def free(self):
        if self.ptr:
            self.array = None
            self._L.qp3d_host_free(self.ptr)
            self.ptr = None

    def __del__(self):
        try:
            self.free()
        except Exception:
            pass


def make_snap(callback, ntsnap, kinds):
    """Wrap a Python callable(step, kind, array) as a qp3d_snap."""
    def _fn(user, step, kind, data, n0, n1, n2):
        try:
            arr = np.ctypeslib.as_array(data, shape=(n0 * n1 * n2,)).copy()
            shape = (n0, n1) if n2 == 1 else (n0, n1, n2)
            return int(callback(step, kind, arr.reshape(shape)) or 0)
        except Exception:
            return 1
    s = Snap()
    s.ntsnap = ntsnap
    s.kinds = sum(1 << k for k in kinds)
    s.fn = SNAP_FN(_fn)
    s.user = None
    s._keep = s.fn
    return s
