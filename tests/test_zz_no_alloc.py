"""The allocation-free likelihood entry point (mrf_likelihood_device_noalloc).

It serves callers that must not allocate device memory while scoring depth
images against a map -- real-time pose-search loops, where cudaMalloc can
stall the device, and hosts whose allocator owns all device memory.  This
file is collected last so that a stop-at-first-failure run has already run
every other test; it passes alone in a fresh process and after the rest.

Checked through the C ABI: two calls in a row against the regular
mrf_likelihood_device on the same map and inputs (also on an 848x480 image,
whose border clip the entry point applies on the fly, and on a map without
active bricks), that repeated calls leave the device's free memory
unchanged, and the size limit."""
import ctypes as C

import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic

pytestmark = pytest.mark.gpu

LIKE_TOL = 1e-3  # per-pixel log-likelihood, absolute (as in the parity tests)


def _fp(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))


def _regular(lib, m, pose, d_depth, hw):
    import torch
    img = torch.zeros(hw, device="cuda")
    s = torch.zeros(1, device="cuda")
    assert lib.mrf_likelihood_device(m.handle, _fp(pose), C.c_void_p(d_depth.data_ptr()),
                                     C.c_void_p(img.data_ptr()), C.c_void_p(s.data_ptr())) == 0
    m.synchronize()
    return img.cpu().numpy(), s.item()


def _noalloc(lib, m, pose, d_depth, img, s):
    st = lib.mrf_likelihood_device_noalloc(m.handle, _fp(pose), C.c_void_p(d_depth.data_ptr()),
                                           C.c_void_p(img.data_ptr()) if img is not None else None,
                                           C.c_void_p(s.data_ptr()))
    assert st == 0, lib.mrf_last_error()
    m.synchronize()


def _check_two_calls(lib, m, pose, depth):
    import torch
    hw = depth.size
    d_depth = torch.from_numpy(np.ascontiguousarray(depth, np.float32)).cuda()
    ref_img, ref_sum = _regular(lib, m, pose, d_depth, hw)
    for _ in range(2):  # two calls in a row share the fixed scratch array
        img = torch.full((hw,), 7.0, device="cuda")
        s = torch.full((1,), 7.0, device="cuda")
        _noalloc(lib, m, pose, d_depth, img, s)
        np.testing.assert_allclose(img.cpu().numpy(), ref_img, atol=LIKE_TOL, rtol=0)
        assert s.item() == pytest.approx(ref_sum, rel=1e-6, abs=1e-3)
    return img.cpu().numpy().reshape(depth.shape)


def test_noalloc_matches_regular_entry_point(native_lib):
    w = synthetic.small_room(5, n_frames=3, rows=90, cols=120)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=4)
    lib = L.load()
    for view in (0, 2):
        depth = w.depths[view].copy()
        depth[::7, ::5] = np.nan          # non-finite returns are cleaned on the fly
        depth[3, :] = np.inf
        img = _check_two_calls(lib, m, w.poses[view], depth)
        # the NaN/inf pixels count as "no return" (likelihood 0)
        assert np.all(img[~np.isfinite(depth)] == 0)
    m.close()


def test_noalloc_848x480_border_clip(native_lib):
    """848x480 images lose a 24/20-pixel border (the reference's clean-up of
    that sensor's images); the entry point applies the same rule on the fly."""
    w = synthetic.small_room(3, n_frames=2, rows=480, cols=848)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=2)
    lib = L.load()
    img = _check_two_calls(lib, m, w.poses[1], w.depths[1])
    border = np.ones(img.shape, bool)
    border[20:-20, 24:-24] = False
    assert np.all(img[border] == 0)
    assert np.any(img[~border] != 0)
    m.close()


def test_noalloc_on_an_empty_map(native_lib):
    """Before any brick is active every pixel with a return scores
    ln(LIKE_EPS), as with the regular entry point."""
    w = synthetic.small_room(1, n_frames=1, rows=60, cols=80)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    lib = L.load()
    img = _check_two_calls(lib, m, w.poses[0], w.depths[0])
    valid = w.depths[0] > 0
    np.testing.assert_allclose(img[valid], np.log(1e-3), rtol=1e-6)
    m.close()


def test_noalloc_leaves_device_memory_untouched(native_lib):
    """After a first call (which looks the scratch array up), further calls
    change nothing in the device's free memory: no allocation on this path."""
    import torch
    w = synthetic.small_room(6, n_frames=2, rows=120, cols=160)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=3)
    lib = L.load()
    hw = w.params.rows * w.params.cols
    d_depth = torch.from_numpy(np.ascontiguousarray(w.depths[0])).cuda()
    img = torch.empty(hw, device="cuda")
    s = torch.empty(1, device="cuda")
    _noalloc(lib, m, w.poses[0], d_depth, img, s)
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info()
    for k in range(20):
        _noalloc(lib, m, w.poses[k % 2], d_depth, img if k % 3 else None, s)
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info()
    assert free1 == free0
    m.close()


def test_noalloc_rejects_images_beyond_the_scratch_limit(native_lib):
    from mrfmap_gb300.params import MapParams
    import torch
    # 800 x 760 = 608,000 pixels > 524,288 (linear sensor polynomials keep
    # the per-tile table within the reference's 3096-float limit)
    p = MapParams(res=0.05, dims=(4.0, 4.0, 3.0), rows=760, cols=800, fx=500.0, fy=500.0,
                  cx=400.0, cy=380.0, prior=0.1)
    p.set_const_polys([0.01, 0.0], [0.0, 0.0], lookup_n=2)
    m = L.MRFMap(p)
    m.load_map(np.array([[40.5, 40.5, 10.5]], np.float32), np.array([0.9], np.float32))
    d_depth = torch.ones(p.rows * p.cols, device="cuda")
    s = torch.zeros(1, device="cuda")
    lib = L.load()
    st = lib.mrf_likelihood_device_noalloc(m.handle, _fp(np.eye(4)), C.c_void_p(d_depth.data_ptr()),
                                           None, C.c_void_p(s.data_ptr()))
    assert st == L.MRF_OK + 1  # MRF_ERR_INVALID
    assert b"524288" in lib.mrf_last_error()
    m.close()
