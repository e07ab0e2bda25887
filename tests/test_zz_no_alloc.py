"""The allocation-free likelihood entry point (mrf_likelihood_device_noalloc).

It serves callers that must not allocate device memory while scoring depth
images against a map -- real-time pose-search loops, where cudaMalloc can
stall the device, and hosts whose allocator owns all device memory.  This
file is collected last so that a stop-at-first-failure run has already run
every other test; it passes alone in a fresh process and after the rest.

Checked through the C ABI: two calls in a row against the regular
mrf_likelihood_device on the same map and inputs, and the size limit."""
import ctypes as C

import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic

pytestmark = pytest.mark.gpu

LIKE_TOL = 1e-3  # per-pixel log-likelihood, absolute (as in the parity tests)


def _fp(a):
    return np.ascontiguousarray(a, np.float32).ctypes.data_as(C.POINTER(C.c_float))


def test_noalloc_matches_regular_entry_point(native_lib):
    import torch
    w = synthetic.small_room(5, n_frames=3, rows=90, cols=120)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=4)
    lib = L.load()
    hw = w.params.rows * w.params.cols
    for view in (0, 2):
        depth = w.depths[view].copy()
        depth[::7, ::5] = np.nan          # non-finite returns are cleaned on the fly
        depth[3, :] = np.inf
        d_depth = torch.from_numpy(depth).cuda()
        ref_img = torch.zeros(hw, device="cuda")
        ref_sum = torch.zeros(1, device="cuda")
        pose = _fp(w.poses[view])
        assert lib.mrf_likelihood_device(m.handle, pose, C.c_void_p(d_depth.data_ptr()),
                                         C.c_void_p(ref_img.data_ptr()),
                                         C.c_void_p(ref_sum.data_ptr())) == 0
        m.synchronize()
        for _ in range(2):  # two calls in a row share the fixed scratch array
            img = torch.full((hw,), 7.0, device="cuda")
            s = torch.full((1,), 7.0, device="cuda")
            st = lib.mrf_likelihood_device_noalloc(m.handle, pose, C.c_void_p(d_depth.data_ptr()),
                                                   C.c_void_p(img.data_ptr()),
                                                   C.c_void_p(s.data_ptr()))
            assert st == 0, lib.mrf_last_error()
            m.synchronize()
            np.testing.assert_allclose(img.cpu().numpy(), ref_img.cpu().numpy(), atol=LIKE_TOL, rtol=0)
            assert s.item() == pytest.approx(ref_sum.item(), rel=1e-6, abs=1e-3)
            # the NaN/inf pixels count as "no return" (likelihood 0)
            assert np.all(img.cpu().numpy().reshape(depth.shape)[~np.isfinite(depth)] == 0)
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
