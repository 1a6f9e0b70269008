"""The allocation-free reduction entry point (frgpu_reduce2d_noalloc).

It serves callers that cannot let the library call cudaMalloc (hosts whose
own memory pool must own every device byte, or processes with a fixed device
footprint): scratch comes from a static device array inside libfrgpu.so, and
the caller passes device inputs and a device output.  Checked through the C
ABI against the allocating entry points frgpu_reduce / frgpu_cfl_dt on the
same state, two calls in a row on meshes of different sizes (so the second
call runs on scratch the first one left behind), within the 1e-13 relative
tolerance the other reduction tests use; in FP64 and in the FP32K form (a
float state with its float low part).  Kept in a file of its own, collected
last.
"""
import ctypes as C
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-13


def _problem(frgpu, nx, ny, deg, amp, precision="fp64"):
    ps = frgpu.FRPSpace2D(0, 1, nx, 0, 1, ny, deg)
    X, Y = ps.xpg[..., 0], ps.xpg[..., 1]
    rho = 1 + amp * np.sin(2 * math.pi * (X + 2 * Y))
    u = np.zeros(X.shape + (4,), order="F")
    u[..., 0] = rho
    u[..., 1] = 0.7 * rho
    u[..., 2] = -0.4 * rho
    u[..., 3] = 1 / 0.4 + 0.5 * rho * (0.49 + 0.16) + 0.1 * np.cos(2 * math.pi * X)
    prob = frgpu.FREuler2DProblem(u, (0, 1), ps, 1.4, flux="lf", bc="period", precision=precision)
    itg = frgpu.init(prob, dt=1e-4)
    sums, speed = itg.reduce()
    rate = 0.1 / itg.cfl_dt(0.1)
    return ps, u, itg, sums, speed, rate


def test_reduce2d_noalloc_matches_allocating_reduce(frgpu):
    import torch

    from frgpu import _lib as L

    lib = L.lib()
    torch.cuda.set_device(0)
    cases = [_problem(frgpu, 96, 80, 3, 0.2), _problem(frgpu, 20, 12, 2, 0.3)]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for ps, u, itg, sums, speed, rate in cases:
        itg.synchronize()
        # the caller's own device array in the reference layout u[i, j, k, l, m]
        state = torch.tensor(np.asarray(u).ravel(order="F"), dtype=torch.float64, device="cuda")
        ptr = C.c_void_p(state.data_ptr())
        wp = torch.tensor(np.asarray(ps.wp).ravel(order="F"), dtype=torch.float64, device="cuda")
        out = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
        L.check(lib.frgpu_reduce2d_noalloc(ptr, None, L.FP64, ps.nx, ps.ny, ps.deg, ps.dx, ps.dy, 1.4,
                                           C.c_void_p(wp.data_ptr()), C.c_void_p(out.data_ptr()), stream))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:4], sums, rtol=RTOL, atol=RTOL * np.abs(sums).max())
        assert abs(got[4] - speed) <= RTOL * speed
        assert abs(got[5] - rate) <= RTOL * rate


def test_reduce2d_noalloc_fp32k_matches_allocating_reduce(frgpu):
    """FP32K: the caller's float state hi = fl(u) and low part lo = fl(u - hi)
    (the split frgpu_state_upload makes) give the sums and wave speeds of
    frgpu_reduce / frgpu_cfl_dt on the FP32K problem of the same state: sums
    within 1e-13 (both accumulate hi + lo as double-float pairs; only the
    partial blocks' order differs), wave speeds (FP32, the same per-point
    arithmetic) within 1e-7."""
    import torch

    from frgpu import _lib as L

    lib = L.lib()
    torch.cuda.set_device(0)
    cases = [_problem(frgpu, 96, 80, 3, 0.2, "fp32k"), _problem(frgpu, 20, 12, 2, 0.3, "fp32k")]
    stream = C.c_void_p(torch.cuda.current_stream().cuda_stream)
    for ps, u, itg, sums, speed, rate in cases:
        itg.synchronize()
        flat = np.asarray(u).ravel(order="F")
        hi = flat.astype(np.float32)
        lo = (flat - hi.astype(np.float64)).astype(np.float32)
        d_hi = torch.tensor(hi, device="cuda")
        d_lo = torch.tensor(lo, device="cuda")
        wp = torch.tensor(np.asarray(ps.wp).ravel(order="F"), dtype=torch.float64, device="cuda")
        out = torch.full((6,), float("nan"), dtype=torch.float64, device="cuda")
        L.check(lib.frgpu_reduce2d_noalloc(C.c_void_p(d_hi.data_ptr()), C.c_void_p(d_lo.data_ptr()), L.FP32K,
                                           ps.nx, ps.ny, ps.deg, ps.dx, ps.dy, 1.4, C.c_void_p(wp.data_ptr()),
                                           C.c_void_p(out.data_ptr()), stream))
        torch.cuda.synchronize()
        got = out.cpu().numpy()
        np.testing.assert_allclose(got[:4], sums, rtol=RTOL, atol=RTOL * np.abs(sums).max())
        assert abs(got[4] - speed) <= 1e-7 * speed
        assert abs(got[5] - rate) <= 1e-7 * rate


def test_reduce2d_noalloc_rejects_meshes_beyond_its_scratch(frgpu):
    from frgpu import _lib as L

    lib = L.lib()
    dummy = C.c_void_p(16)  # never dereferenced: the argument checks come first
    rc = lib.frgpu_reduce2d_noalloc(dummy, None, L.FP64, 8192, 8192, 3, 1e-4, 1e-4, 1.4, dummy, dummy, None)
    assert rc == L.ERR_ARG
    assert "exceed the maximum" in L.last_error()
    # below 67,108,864 points, but ceil(1,851,393 / 16384) * 36 = 4104 blocks > 4096
    rc = lib.frgpu_reduce2d_noalloc(dummy, None, L.FP64, 1851393, 1, 5, 1e-4, 1e-4, 1.4, dummy, dummy, None)
    assert rc == L.ERR_ARG
    assert "4104 partial blocks" in L.last_error()
    # a low part belongs to the FP32K form only
    rc = lib.frgpu_reduce2d_noalloc(dummy, dummy, L.FP64, 8, 8, 3, 1e-4, 1e-4, 1.4, dummy, dummy, None)
    assert rc == L.ERR_ARG
    assert "d_lo must be NULL" in L.last_error()


def test_device_state_has_the_documented_2d_layout(frgpu):
    """frgpu_problem_device_state hands out the 2D Euler state in the device
    layout include/frgpu.h documents: value (i, j, k, l, m) at
    ((k + np l) nx ny + i + nx j) 4 + m."""
    import torch

    from frgpu import _lib as L

    ps, u, itg, *_ = _problem(frgpu, 24, 10, 3, 0.2)
    itg.synchronize()
    ptr, eb = C.c_void_p(), C.c_int()
    L.check(L.lib().frgpu_problem_device_state(itg.prob._h, C.byref(ptr), C.byref(eb)))
    assert eb.value == 8
    n = u.size

    class _Dev:
        __cuda_array_interface__ = {"shape": (n,), "typestr": "<f8", "data": (ptr.value, False), "version": 3}

    dev = torch.as_tensor(_Dev(), device="cuda").cpu().numpy()
    npp = ps.deg + 1
    want = np.transpose(np.asarray(u).reshape(ps.nx, ps.ny, npp * npp, 4, order="F"), (2, 1, 0, 3)).ravel()
    np.testing.assert_array_equal(dev, want)
