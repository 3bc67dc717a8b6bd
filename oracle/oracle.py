"""ctypes bindings for the CPU oracle (test infrastructure only).

Only tests/, ``__graft_entry__.smoke()`` and the CPU-baseline leg of bench.py
import this module, and only as the checker.  It never stands in for the CUDA
path.
"""
import ctypes
import os

import numpy as np

from . import build as _build

REF32, F64, MIRROR = 0, 1, 2

_f32p = ctypes.POINTER(ctypes.c_float)


class OracleArgs(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("pml", ctypes.c_int), ("sz", ctypes.c_int),
        ("dx", ctypes.c_float), ("dy", ctypes.c_float), ("dz", ctypes.c_float),
        ("dt", ctypes.c_float),
        ("vp", _f32p), ("epsilon", _f32p), ("delta", _f32p),
        ("source", _f32p), ("wavelet", _f32p),
        ("dlr", _f32p), ("ddlr", _f32p), ("dtb", _f32p), ("ddtb", _f32p),
        ("dfb", _f32p), ("ddfb", _f32p),
        ("c", _f32p), ("c2", _f32p),
        ("nthreads", ctypes.c_int), ("live", ctypes.c_int),
    ]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        path = _build.LIB
        if not os.path.exists(path):
            _build.build_oracle()
        _lib = ctypes.CDLL(path)
        _lib.oracle_run.restype = ctypes.c_int
        _lib.oracle_run.argtypes = [ctypes.c_int, ctypes.POINTER(OracleArgs),
                                    ctypes.c_int, ctypes.c_int] + [ctypes.c_void_p] * 6
        _lib.oracle_pml_state_size.restype = ctypes.c_size_t
        _lib.oracle_pml_state_size.argtypes = [ctypes.c_int] * 4
        _lib.oracle_threshold_f.restype = ctypes.c_float
        _lib.oracle_threshold_f.argtypes = [ctypes.c_float]
        _lib.oracle_threshold_m2.restype = ctypes.c_float
        _lib.oracle_threshold_m2.argtypes = [ctypes.c_float]
        _lib.oracle_absmax.restype = ctypes.c_float
        _lib.oracle_absmax.argtypes = [ctypes.c_void_p, ctypes.c_size_t]
        for name in ("oracle_fdcoff1", "oracle_fdcoff2"):
            getattr(_lib, name).argtypes = [ctypes.c_void_p]
        _lib.oracle_pmlcoff.argtypes = ([ctypes.c_int] + [ctypes.c_float] * 4 +
                                        [ctypes.c_void_p] * 6)
        _lib.oracle_source.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_float] * 8 +
                                       [ctypes.c_int] * 4 + [ctypes.c_void_p] * 2)
        _lib.oracle_extend_model.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 4
    return _lib


def ref_lib():
    """The reference's own CPU operators, or None where they were not built."""
    global _ref
    if _ref is None:
        path = _build.REF_LIB
        if not os.path.exists(path):
            path = _build.build_reference()
            if path is None:
                return None
        _ref = ctypes.CDLL(path)
        _ref.ref_run.restype = ctypes.c_int
        _ref.ref_run.argtypes = ([ctypes.c_int] * 5 + [ctypes.c_float] * 4 +
                                 [ctypes.c_void_p] * 13 + [ctypes.c_int] * 2 +
                                 [ctypes.c_void_p] * 6)
        _ref.ref_pml_state_size.restype = ctypes.c_size_t
        _ref.ref_pml_state_size.argtypes = [ctypes.c_int] * 4
        _ref.ref_fdcoff.argtypes = [ctypes.c_void_p] * 2
        _ref.ref_pmlcoff.argtypes = [ctypes.c_int] + [ctypes.c_float] * 4 + [ctypes.c_void_p] * 6
        _ref.ref_source.argtypes = ([ctypes.c_int] * 3 + [ctypes.c_float] * 8 +
                                    [ctypes.c_int] * 4 + [ctypes.c_void_p] * 2)
        _ref.ref_extend_model.argtypes = [ctypes.c_void_p, ctypes.c_void_p] + [ctypes.c_int] * 4
        _ref.ref_absmax.restype = ctypes.c_float
        _ref.ref_absmax.argtypes = [ctypes.c_void_p] + [ctypes.c_int] * 3
    return _ref


def _ptr(a):
    return a.ctypes.data_as(ctypes.c_void_p) if a is not None else None


def _fp(a):
    return a.ctypes.data_as(_f32p) if a is not None else None


def pml_state_size(nx, ny, nz, pml):
    return int(lib().oracle_pml_state_size(nx, ny, nz, pml))


def fdcoff():
    c = np.zeros(36, np.float32)
    c2 = np.zeros(36, np.float32)
    lib().oracle_fdcoff1(_ptr(c))
    lib().oracle_fdcoff2(_ptr(c2))
    return c, c2


def pmlcoff(pml, vpmax, dx, dy, dz):
    out = [np.zeros(max(pml, 1), np.float32) for _ in range(6)]
    lib().oracle_pmlcoff(pml, vpmax, dx, dy, dz, *[_ptr(o) for o in out])
    return out  # dlr, ddlr, dtb, ddtb, dfb, ddfb


def source(sx, sy, sz, fm, amp, alpha, dt, dx, dy, dz, t0, nt, nx, ny, nz):
    src = np.zeros(nx * ny * nz, np.float32)
    wav = np.zeros(nt, np.float32)
    lib().oracle_source(sx, sy, sz, fm, amp, alpha, dt, dx, dy, dz, t0, nt,
                        nx, ny, nz, _ptr(src), _ptr(wav))
    return src, wav


def extend_model(interior, nx, ny, nz, pml):
    out = np.zeros(nx * ny * nz, np.float32)
    inp = np.ascontiguousarray(interior, np.float32).ravel()
    lib().oracle_extend_model(_ptr(inp), _ptr(out), nx, ny, nz, pml)
    return out


def threshold_m2(uxyzmax):
    return float(lib().oracle_threshold_m2(float(uxyzmax)))


def threshold_f(uxyzmax):
    return float(lib().oracle_threshold_f(float(uxyzmax)))


class Problem:
    """One shot's inputs in the reference's padded layout ([nz][nx][ny])."""

    def __init__(self, nx, ny, nz, pml, sz, dx, dy, dz, dt, vp, eps, delta,
                 src, wavelet, prof, c, c2):
        self.nx, self.ny, self.nz, self.pml, self.sz = nx, ny, nz, pml, sz
        self.dx, self.dy, self.dz, self.dt = dx, dy, dz, dt
        f = lambda a: np.ascontiguousarray(a, np.float32).ravel()
        self.vp, self.eps, self.delta = f(vp), f(eps), f(delta)
        self.src = None if src is None else f(src)
        self.wavelet = f(wavelet)
        self.prof = [f(p) for p in prof]
        self.c, self.c2 = f(c), f(c2)

    @property
    def N(self):
        return self.nx * self.ny * self.nz

    @property
    def nt(self):
        return len(self.wavelet)

    def to_oracle(self, O=None):
        """Already an oracle problem (the library's Shot converts itself)."""
        return self

    def args(self, nthreads=0):
        a = OracleArgs()
        a.nx, a.ny, a.nz, a.pml, a.sz = self.nx, self.ny, self.nz, self.pml, self.sz
        a.dx, a.dy, a.dz, a.dt = self.dx, self.dy, self.dz, self.dt
        a.vp, a.epsilon, a.delta = _fp(self.vp), _fp(self.eps), _fp(self.delta)
        a.source, a.wavelet = _fp(self.src), _fp(self.wavelet)
        (a.dlr, a.ddlr, a.dtb, a.ddtb, a.dfb, a.ddfb) = [_fp(p) for p in self.prof]
        a.c, a.c2 = _fp(self.c), _fp(self.c2)
        a.nthreads = nthreads
        return a


class State:
    """u1, u2, u3 and the canonical PML state of one shot."""

    def __init__(self, prob, dtype=np.float32):
        n = prob.N
        self.u1 = np.zeros(n, dtype)
        self.u2 = np.zeros(n, dtype)
        self.u3 = np.zeros(n, dtype)
        self.pml = np.zeros(pml_state_size(prob.nx, prob.ny, prob.nz, prob.pml) + 1, dtype)

    def copy(self, dtype=None):
        s = State.__new__(State)
        for k in ("u1", "u2", "u3", "pml"):
            v = getattr(self, k)
            setattr(s, k, v.astype(dtype) if dtype is not None else v.copy())
        return s


def run(variant, prob, k0=0, nsteps=None, state=None, nthreads=0,
        want_record=True):
    """Advance ``state`` (created if None) by nsteps; returns (record, uxyzmax, state)."""
    if nsteps is None:
        nsteps = prob.nt - k0
    dt = np.float64 if variant == F64 else np.float32
    if state is None:
        state = State(prob, dt)
    hx, hy = prob.nx - 2 * prob.pml, prob.ny - 2 * prob.pml
    rec = np.zeros((nsteps, hx, hy), dt) if want_record else None
    mx = np.zeros(nsteps, dt)
    args = prob.args(nthreads)
    rc = lib().oracle_run(variant, ctypes.byref(args), k0, nsteps,
                          _ptr(state.u1), _ptr(state.u2), _ptr(state.u3),
                          _ptr(state.pml), _ptr(rec), _ptr(mx))
    if rc != 0:
        raise RuntimeError("oracle_run failed: %d" % rc)
    return rec, mx, state


def run_reference(prob, k0=0, nsteps=None, state=None):
    """Same as run(REF32, ...) but through the reference's own CPU operators."""
    rl = ref_lib()
    if rl is None:
        raise RuntimeError("reference CPU operators were not built here")
    if nsteps is None:
        nsteps = prob.nt - k0
    if state is None:
        state = State(prob, np.float32)
    hx, hy = prob.nx - 2 * prob.pml, prob.ny - 2 * prob.pml
    rec = np.zeros((nsteps, hx, hy), np.float32)
    mx = np.zeros(nsteps, np.float32)
    p = prob
    rc = rl.ref_run(p.nx, p.ny, p.nz, p.pml, p.sz, p.dx, p.dy, p.dz, p.dt,
                    _ptr(p.vp), _ptr(p.eps), _ptr(p.delta), _ptr(p.src),
                    _ptr(p.wavelet), *[_ptr(q) for q in p.prof], _ptr(p.c),
                    _ptr(p.c2), k0, nsteps, _ptr(state.u1), _ptr(state.u2),
                    _ptr(state.u3), _ptr(state.pml), _ptr(rec), _ptr(mx))
    if rc != 0:
        raise RuntimeError("ref_run failed: %d" % rc)
    return rec, mx, state


_refgpu = None


def ref_gpu_available():
    """True when the reference GPU kernels were compiled (a cubin exists)."""
    return os.path.exists(_build.REF_CUBIN)


def ref_gpu_lib():
    """Host driver of the reference's own GPU kernels (ref_gpu.cu), with the
    reference cubin loaded; None when the cubin was not built."""
    global _refgpu
    if _refgpu is None:
        if not ref_gpu_available():
            return None
        _build.build_reference_gpu()
        L = ctypes.CDLL(_build.REFGPU_LIB)
        L.refgpu_load.restype = ctypes.c_int
        L.refgpu_load.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
        L.refgpu_run.restype = ctypes.c_int
        L.refgpu_run.argtypes = ([ctypes.POINTER(OracleArgs), ctypes.c_int, ctypes.c_int] +
                                 [ctypes.c_void_p] * 6 + [ctypes.c_int,
                                 ctypes.POINTER(ctypes.c_double), ctypes.c_char_p,
                                 ctypes.c_size_t])
        err = ctypes.create_string_buffer(512)
        if L.refgpu_load(_build.REF_CUBIN.encode(), err, len(err)) != 0:
            raise RuntimeError("reference GPU kernels: " + err.value.decode())
        _refgpu = L
    return _refgpu


def run_reference_gpu(prob, k0=0, nsteps=None, state=None, host_max=False, want_record=True):
    """The reference's own GPU kernels (GPU_kernel.cu built for sm_103a) on
    cuda:0, in the reference GPU driver's step sequence; returns (record,
    uxyzmax, state, ms) with ms the wall time of the time loop.  host_max:
    take each step's max on the host from full copies, as the reference's
    driver does, instead of a device reduction (same values)."""
    L = ref_gpu_lib()
    if L is None:
        raise RuntimeError("reference GPU kernels were not built")
    if nsteps is None:
        nsteps = prob.nt - k0
    if state is None:
        state = State(prob, np.float32)
    hx, hy = prob.nx - 2 * prob.pml, prob.ny - 2 * prob.pml
    rec = np.zeros((nsteps, hx, hy), np.float32) if want_record else None
    mx = np.zeros(nsteps, np.float32)
    ms = ctypes.c_double(0.0)
    err = ctypes.create_string_buffer(512)
    args = prob.args()
    rc = L.refgpu_run(ctypes.byref(args), k0, nsteps, _ptr(state.u1), _ptr(state.u2),
                      _ptr(state.u3), _ptr(state.pml), _ptr(rec), _ptr(mx), int(host_max),
                      ctypes.byref(ms), err, len(err))
    if rc != 0:
        raise RuntimeError("refgpu_run failed: " + err.value.decode())
    return rec, mx, state, ms.value


# ---------------------------------------------------------------------------
# FP64 adjoint (qp3d_adjoint.c)
# ---------------------------------------------------------------------------
_f64p = ctypes.POINTER(ctypes.c_double)


class AdjArgs(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("pml", ctypes.c_int), ("sz", ctypes.c_int), ("nt", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double),
        ("dt", ctypes.c_double),
        ("vp", _f64p), ("eps", _f64p), ("del_", _f64p),
        ("source", _f32p), ("wavelet", _f32p),
        ("dlr", _f32p), ("ddlr", _f32p), ("dtb", _f32p), ("ddtb", _f32p),
        ("dfb", _f32p), ("ddfb", _f32p),
        ("c", _f32p), ("c2", _f32p),
        ("nthreads", ctypes.c_int), ("live", ctypes.c_int),
    ]


def _adj_lib():
    L = lib()
    if not getattr(L, "_adj_ready", False):
        P = ctypes.POINTER(AdjArgs)
        L.oracle_adj_freeze.argtypes = [P, ctypes.c_void_p, ctypes.c_void_p]
        L.oracle_adj_forward.argtypes = [P] + [ctypes.c_void_p] * 5
        L.oracle_adj_backward.argtypes = [P] + [ctypes.c_void_p] * 8
        L.oracle_adj_tlm.argtypes = [P] + [ctypes.c_void_p] * 5
        for f in (L.oracle_adj_freeze, L.oracle_adj_forward, L.oracle_adj_backward,
                  L.oracle_adj_tlm):
            f.restype = ctypes.c_int
        L._adj_ready = True
    return L


class Adjoint:
    """FP64 frozen-operator forward and adjoint of one problem.  The model is
    held in double (vp, eps, delta as float64 arrays of N cells) so finite
    differences can perturb it; the scalar operator is frozen by freeze()."""

    def __init__(self, prob, source=True, nthreads=0, live=False):
        self.p = prob
        self.vp = prob.vp.astype(np.float64)
        self.eps = prob.eps.astype(np.float64)
        self.delta = prob.delta.astype(np.float64)
        self.use_source = source
        self.nthreads = nthreads
        self.live = live          # backward: S's dependence on grad u included
        self.fa = self.fb = None

    def _args(self, vp=None, eps=None, delta=None):
        p = self.p
        self._keep = [np.ascontiguousarray(v if v is not None else d, np.float64)
                      for v, d in ((vp, self.vp), (eps, self.eps), (delta, self.delta))]
        a = AdjArgs()
        a.nx, a.ny, a.nz, a.pml, a.sz, a.nt = p.nx, p.ny, p.nz, p.pml, p.sz, p.nt
        a.dx, a.dy, a.dz, a.dt = p.dx, p.dy, p.dz, p.dt
        a.vp, a.eps, a.del_ = [k.ctypes.data_as(_f64p) for k in self._keep]
        a.source = _fp(p.src) if (self.use_source and p.src is not None) else None
        a.wavelet = _fp(p.wavelet)
        a.dlr, a.ddlr, a.dtb, a.ddtb, a.dfb, a.ddfb = [_fp(x) for x in p.prof]
        a.c, a.c2 = _fp(p.c), _fp(p.c2)
        a.nthreads = self.nthreads
        a.live = 1 if self.live else 0
        return a

    def freeze(self, with_source=True):
        """Frozen factors from a base run (the live operator), by default with
        the problem's source even when the adjoint runs without it."""
        n = self.p.N * self.p.nt
        self.fa = np.zeros(n, np.float64)
        self.fb = np.zeros(n, np.float64)
        keep, self.use_source = self.use_source, with_source
        a = self._args()
        self.use_source = keep
        rc = _adj_lib().oracle_adj_freeze(ctypes.byref(a), _ptr(self.fa), _ptr(self.fb))
        assert rc == 0, rc
        return self

    def live_forward(self, vp=None, eps=None, delta=None):
        """Record of the live operator (S from the run's own wavefield) at the
        given model: factors frozen on that model, then the run with them."""
        n = self.p.N * self.p.nt
        fa = np.zeros(n, np.float64)
        fb = np.zeros(n, np.float64)
        a = self._args(vp, eps, delta)
        rc = _adj_lib().oracle_adj_freeze(ctypes.byref(a), _ptr(fa), _ptr(fb))
        assert rc == 0, rc
        keep = self.fa, self.fb
        self.fa, self.fb = fa, fb
        try:
            return self.forward(vp=vp, eps=eps, delta=delta)
        finally:
            self.fa, self.fb = keep

    def forward(self, extra=None, want_hist=False, vp=None, eps=None, delta=None):
        p = self.p
        rec = np.zeros((p.nt, p.nx - 2 * p.pml, p.ny - 2 * p.pml), np.float64)
        hist = np.zeros(p.N * p.nt, np.float64) if want_hist else None
        a = self._args(vp, eps, delta)
        ex = None if extra is None else np.ascontiguousarray(extra, np.float64).ravel()
        rc = _adj_lib().oracle_adj_forward(ctypes.byref(a), _ptr(self.fa), _ptr(self.fb),
                                           _ptr(ex), _ptr(rec), _ptr(hist))
        assert rc == 0, rc
        return (rec, hist) if want_hist else rec

    def tlm(self, hist, extra):
        """Records of the tangent-linear response to additive sources extra
        (nt x N) about the base trajectory hist (from forward(want_hist=True));
        with live, S's perturbation through the unit normal is included."""
        p = self.p
        rec = np.zeros((p.nt, p.nx - 2 * p.pml, p.ny - 2 * p.pml), np.float64)
        a = self._args()
        ex = np.ascontiguousarray(extra, np.float64).ravel()
        rc = _adj_lib().oracle_adj_tlm(ctypes.byref(a), _ptr(self.fa), _ptr(self.fb),
                                       _ptr(hist), _ptr(ex), _ptr(rec))
        assert rc == 0, rc
        return rec

    def backward(self, hist, resid, want_fadj=False):
        p = self.p
        g = [np.zeros(p.N, np.float64) for _ in range(3)]
        fadj = np.zeros(p.N * p.nt, np.float64) if want_fadj else None
        a = self._args()
        r = np.ascontiguousarray(resid, np.float64).ravel()
        rc = _adj_lib().oracle_adj_backward(ctypes.byref(a), _ptr(self.fa), _ptr(self.fb),
                                            _ptr(hist), _ptr(r), _ptr(g[0]), _ptr(g[1]),
                                            _ptr(g[2]), _ptr(fadj))
        assert rc == 0, rc
        return (g, fadj) if want_fadj else g
