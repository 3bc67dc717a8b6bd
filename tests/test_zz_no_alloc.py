"""qp3d_gradmax_noalloc: max|grad u| without any device allocation (GPU).

Callers that cannot let a library allocate device memory -- a framework that
already holds the whole device in its own pool, or a loop that must not
allocate after start-up -- use this entry point with a wavefield they keep in
device memory.  Its scratch is a fixed device array shared by all calls.  The
test allocates the input and output itself (with torch, as such a caller
would), calls the entry point through the C ABI twice in a row, and checks
both results against the library's ordinary path, which computes the same
maximum for the step that starts from this wavefield, and that the device's
free memory does not change across the calls.  A device wait that runs out
(test hook: a plane that is never loaded) is reported as QP3D_ERR_TIMEOUT,
and the next call works.  Collected last on purpose.
"""
import ctypes

import numpy as np
import pytest

import qp3d
import synthetic

pytestmark = pytest.mark.gpu


def _device_copy(torch, vol, nz, nx, ny, ldy):
    """[nz][nx][ny] host volume -> [nz][nx][ldy] device tensor (caller-owned)."""
    host = np.zeros((nz, nx, ldy), np.float32)
    host[:, :, :ny] = vol.reshape(nz, nx, ny)
    return torch.from_numpy(host).cuda()


@pytest.mark.parametrize("hx,hy,nz0,pml,steps", [(22, 24, 18, 8, 40), (27, 21, 30, 10, 55)])
def test_gradmax_noalloc_matches_the_library_path(ctx, hx, hy, nz0, pml, steps):
    torch = pytest.importorskip("torch")
    shot = synthetic.small_case(hx=hx, hy=hy, nz0=nz0, pml=pml, nt=steps + 1, seed=31)
    ctx.load(shot)
    ctx.advance(steps)
    _, u_cur, _ = ctx.read_state()          # u(steps)
    ctx.advance(1)                          # step `steps` computes max|grad u(steps)|
    want = ctx.uxyzmax(steps, 1)[0]
    assert want > 0

    nx, ny, nz = shot.nx, shot.ny, shot.nz
    ldy = (ny + 3) // 4 * 4
    d_u = _device_copy(torch, u_cur, nz, nx, ny, ldy)
    d_max = torch.full((1,), -1.0, dtype=torch.float32, device="cuda")
    L = qp3d.load()
    err = ctypes.create_string_buffer(256)
    got, free = [], []
    for _ in range(3):                      # calls in a row share the scratch
        d_max.fill_(-1.0)
        torch.cuda.synchronize()
        free.append(torch.cuda.mem_get_info()[0])
        rc = _call(L, d_u, nx, ny, nz, ldy, shot, d_max, err)
        assert rc == 0, err.value.decode()
        torch.cuda.synchronize()
        got.append(np.float32(d_max.item()))
    free.append(torch.cuda.mem_get_info()[0])
    # the same arithmetic as the library's path: equal bit for bit
    assert got[0].view(np.uint32) == np.float32(want).view(np.uint32), (got, want)
    assert got[1].view(np.uint32) == got[0].view(np.uint32)
    assert got[2].view(np.uint32) == got[0].view(np.uint32)
    # nothing allocated on the device once the first call has set up its
    # scratch addresses
    assert free[1] == free[2] == free[3], free


def _call(L, d_u, nx, ny, nz, ldy, shot, d_max, err):
    return L.qp3d_gradmax_noalloc(ctypes.c_void_p(d_u.data_ptr()), nx, ny, nz, ldy,
                                  shot.dx, shot.dy, shot.dz,
                                  shot.c.ctypes.data_as(ctypes.c_void_p),
                                  ctypes.c_void_p(d_max.data_ptr()), None, err, len(err))


def test_gradmax_noalloc_reports_a_wait_that_ran_out():
    """A plane that the first CTA never loads (test hook) makes its bounded
    waits run out after 20 ms: the call returns QP3D_ERR_TIMEOUT with NaN in
    the output; with the hook cleared the next call returns the maximum."""
    torch = pytest.importorskip("torch")
    shot = synthetic.small_case(hx=30, hy=26, nz0=24, pml=8, nt=4, seed=3)
    u_prev, u_cur, _ = synthetic.random_state(shot, seed=3)
    nx, ny, nz = shot.nx, shot.ny, shot.nz
    ldy = (ny + 3) // 4 * 4
    d_u = _device_copy(torch, u_cur, nz, nx, ny, ldy)
    d_max = torch.zeros(1, dtype=torch.float32, device="cuda")
    L = qp3d.load()
    err = ctypes.create_string_buffer(256)
    assert _call(L, d_u, nx, ny, nz, ldy, shot, d_max, err) == 0
    want = float(d_max.item())
    try:
        assert L.qp3d_tune(None, b"noalloc_wait_limit_us", 20000) == 0
        assert L.qp3d_tune(None, b"noalloc_test_hold_plane", 2) == 0
        rc = _call(L, d_u, nx, ny, nz, ldy, shot, d_max, err)
        assert rc == -4, (rc, err.value)
        assert b"timed out" in err.value
        assert np.isnan(d_max.item())
    finally:
        L.qp3d_tune(None, b"noalloc_test_hold_plane", -1)
        L.qp3d_tune(None, b"noalloc_wait_limit_us", 0)
    d_max.fill_(-1.0)
    assert _call(L, d_u, nx, ny, nz, ldy, shot, d_max, err) == 0
    assert float(d_max.item()) == want


def test_gradmax_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    L = qp3d.load()
    c = np.zeros(36, np.float32)
    d = torch.zeros(16 * 16 * 16, dtype=torch.float32, device="cuda")
    out = torch.zeros(1, dtype=torch.float32, device="cuda")
    err = ctypes.create_string_buffer(256)
    ptr = ctypes.c_void_p(d.data_ptr())
    optr = ctypes.c_void_p(out.data_ptr())
    cp = c.ctypes.data_as(ctypes.c_void_p)
    # pitch not a multiple of 4
    assert L.qp3d_gradmax_noalloc(ptr, 16, 15, 16, 15, 10.0, 10.0, 10.0, cp, optr, None,
                                  err, len(err)) == -1
    assert b"pitch" in err.value
    # grid beyond the scratch array (70000 x 70000 cells per plane)
    assert L.qp3d_gradmax_noalloc(ptr, 70000, 70000, 16, 70000, 10.0, 10.0, 10.0, cp, optr,
                                  None, err, len(err)) == -1
    assert b"at most" in err.value
    # one tile across y, more than 65535 tiles along x: within the scratch
    # array but beyond the launch grid's second dimension
    assert L.qp3d_gradmax_noalloc(ptr, 65536 * 32 + 10, 16, 16, 16, 10.0, 10.0, 10.0, cp, optr,
                                  None, err, len(err)) == -1
    assert b"65535" in err.value
