"""Evaluation renders (expected depth, accuracy, simple accuracy, occupancy
threshold) on the GPU against the oracle's renders over the same belief
field, and the reference-named entry points of the Python module."""
import os
import sys

import numpy as np
import pytest

from mrfmap_gb300 import _build
from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def inferred(native_lib):
    w = synthetic.small_room(5, n_frames=3, rows=60, cols=80)
    m = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    for P, D in zip(w.poses, w.depths):
        m.add_view(P, D)
    m.infer(iters=4)
    om = O.OracleMap(w.params, threads=4)
    for P, D in zip(w.poses, w.depths):
        om.add_view(P, D, O.ACT_FULL_RAY)
    assert om.num_bricks == m.num_bricks
    om.set_beliefs(m.beliefs())  # same field: the renders alone are compared
    return w, m, om


def _poses(w):
    P = w.poses[1].copy()
    P[0, 3] += 0.07
    return [w.poses[0], w.poses[2], P]


@pytest.mark.parametrize("mode,thresh", [(1, 0.0), (2, 0.5), (2, 0.8), (3, 0.1), (3, 0.5)])
def test_label_renders_match_oracle(inferred, mode, thresh):
    w, m, om = inferred
    for i, P in enumerate(_poses(w)):
        D = w.depths[min(i, 2)]
        img, score, cnt = m.render(mode, P, D, thresh)
        ref, rcnt = om.render(mode, P, D, thresh)
        agree = np.mean(img == ref)
        assert agree >= 0.995, (mode, thresh, i, agree)
        assert cnt.sum() == img.size
        np.testing.assert_array_equal(cnt, [(img == k).sum() for k in (-1, 0, 1, 2)])
        assert np.abs(cnt - rcnt).sum() <= 0.01 * img.size
        if mode == 1:
            assert score == pytest.approx(cnt[2] / max(img.size - cnt[0], 1), rel=1e-6)
        if mode == 2:
            assert score == pytest.approx((cnt[2] + cnt[0]) / img.size, rel=1e-6)


def test_expected_depth_matches_oracle(inferred):
    w, m, om = inferred
    for i, P in enumerate(_poses(w)):
        img, _, _ = m.render(L.RENDER_EXPECTED_DEPTH, P, w.depths[0])
        ref, _ = om.render(0, P, w.depths[0], 0.0)
        hit = ref > 0.05
        assert hit.mean() > 0.5
        np.testing.assert_allclose(img[hit], ref[hit], rtol=2e-3, atol=2e-3)


def test_expected_depth_tracks_measured_depth(inferred):
    """Where the map is confident the expected depth is near the camera's
    z-depth of the measured surface."""
    w, m, _ = inferred
    img, _, _ = m.render_view(L.RENDER_EXPECTED_DEPTH, 0)
    D = w.depths[0]
    ok = np.isfinite(D) & (D > 0.3) & (D < 4.0)
    err = np.abs(img[ok] - D[ok])
    assert np.median(err) < 0.1


def test_render_view_equals_render_at_pose(inferred):
    w, m, _ = inferred
    for mode in range(4):
        a = m.render_view(mode, 2, 0.3)
        b = m.render(mode, w.poses[2], w.depths[2], 0.3)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[2], b[2])


def test_render_errors(inferred):
    w, m, _ = inferred
    with pytest.raises(L.MrfError):
        m.render(7, w.poses[0], w.depths[0])
    with pytest.raises(L.MrfError):
        m.render_view(0, 99)


def test_python_module_render_names(inferred):
    w, m, _ = inferred
    path = _build.build_pymodule()
    sys.path.insert(0, os.path.dirname(path))
    import GVDBPyModules as G
    gp = G.gvdb_params()
    p = w.params
    gp.res, gp.prior, gp.rows, gp.cols = p.res, p.prior, p.rows, p.cols
    gp.dims = list(p.dims)
    gp.K = p.K
    gp.max_iters = p.max_iters
    gp.lookup_n = 3
    gp.const_sigmasq_poly = list(p.const_sigmasq_poly)
    gp.populate_lookup_tables()
    gp.set_from_python()
    inf = G.GVDBInference(True, False)
    for P, D in zip(w.poses, w.depths):
        inf.add_camera_with_depth(P, D)
    inf.perform_inference()
    mm = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        mm.add_view(P, D)
    mm.infer()
    out = np.zeros((p.rows, p.cols), np.float32)
    inf.get_expected_depth_image(1, out)
    np.testing.assert_array_equal(out, mm.render_view(0, 1)[0])
    acc = inf.get_accuracy_image_at_pose(w.poses[0], G.GVDBImage(w.depths[0]), out)
    img, s, _ = mm.render(1, w.poses[0], w.depths[0])
    np.testing.assert_array_equal(out, img)
    assert acc == s

    cen, bel = mm.read_bricks()
    local = np.stack(np.meshgrid(np.arange(8), np.arange(8), np.arange(8), indexing="ij"), -1).reshape(512, 3)
    pts = ((cen[:, None, :] - 4) + local[None] + 0.5).reshape(-1, 3).astype(np.float32)
    occ = bel.reshape(-1)
    keep = occ > 0
    est = G.GVDBMapLikelihoodEstimator(gp, False)
    est.load_map(pts[keep], occ[keep])
    est.set_acc_thresh(0.6)
    a1 = est.get_simple_accuracy_image_at_pose_with_depth(w.poses[0], w.depths[0], out)
    a2 = est.get_simple_accuracy_at_pose(w.poses[0], G.GVDBImage(w.depths[0]))
    assert a1 == a2 and 0.0 <= a1 <= 1.0
    assert set(np.unique(out)) <= {-1.0, 0.0, 1.0, 2.0}
    est.get_occ_thresh_image_at_pose(w.poses[0], G.GVDBImage(w.depths[0]), out, 0.4)
    assert set(np.unique(out)) <= {-1.0, 0.0, 1.0}
    est.add_camera(w.poses[0], G.GVDBImage(w.depths[0]))
    out2 = np.zeros_like(out)
    est.get_accuracy_image(0, out2)
    a3 = est.get_accuracy_image_at_pose_with_depth(w.poses[0], w.depths[0], out)
    np.testing.assert_array_equal(out, out2)
    assert 0.0 <= a3 <= 1.0


def test_pixel_diagnostics_match_oracle_trace(inferred):
    """The per-voxel records of one pixel's ray (the reference's diagnostic
    probe) follow the oracle's traversal bit for bit; visibility and first
    return density follow from the beliefs along it."""
    w, m, om = inferred
    bel = m.beliefs().reshape(-1)
    for (x, y), P in (((40, 30), w.poses[0]), ((5, 52), w.poses[1]), ((77, 3), w.poses[2])):
        d = m.pixel_diagnostics(P, x, y)
        vox, ln, s = om.trace_pixel(P, x, y)
        assert len(d["s"]) == len(vox) > 0
        np.testing.assert_array_equal(d["vox"].astype(np.int64), vox.astype(np.int64))
        np.testing.assert_array_equal(d["s"].view(np.uint32), s.view(np.uint32))
        np.testing.assert_array_equal(d["belief"], bel[vox])
        np.testing.assert_array_equal(d["slot"], vox // 512)
        loc = vox % 512
        np.testing.assert_array_equal(d["local"], np.stack([loc // 64, (loc // 8) % 8, loc % 8], 1))
        A = np.cumsum(np.log1p(-bel[vox].astype(np.float64)) * ln)
        V = np.exp(A)
        np.testing.assert_allclose(d["vis"], V, rtol=1e-4, atol=1e-7)
        Vp = np.concatenate([[1.0], V[:-1]])
        # w = (V_prev - V) / l in fp32: the difference of two visibilities near
        # 1 keeps a few ulps of 1 in absolute terms
        np.testing.assert_allclose(d["w"] * ln, Vp - V, rtol=1e-3, atol=5e-7)
    # a short buffer keeps the first records and says how many it kept
    d = m.pixel_diagnostics(w.poses[0], 40, 30, n_floats=41)
    assert len(d["s"]) == 4
    with pytest.raises(L.MrfError):
        m.pixel_diagnostics(w.poses[0], w.params.cols, 0)


def test_python_module_diagnostics(inferred):
    w, m, _ = inferred
    path = _build.build_pymodule()
    sys.path.insert(0, os.path.dirname(path))
    import GVDBPyModules as G
    p = w.params
    gp = G.gvdb_params()
    gp.res, gp.prior, gp.rows, gp.cols = p.res, p.prior, p.rows, p.cols
    gp.dims = list(p.dims)
    gp.K = p.K
    gp.max_iters = p.max_iters
    gp.lookup_n = 3
    gp.const_sigmasq_poly = list(p.const_sigmasq_poly)
    gp.populate_lookup_tables()
    gp.set_from_python()
    inf = G.GVDBInference(True, False)
    for P, D in zip(w.poses, w.depths):
        inf.add_camera_with_depth(P, D)
    inf.perform_inference()
    mm = L.MRFMap(w.params)
    for P, D in zip(w.poses, w.depths):
        mm.add_view(P, D)
    mm.infer()
    inf.set_selected_x_y(40, 30)
    out = np.zeros((p.rows, p.cols), np.float32)
    inf.get_diagnostic_image(1, out)
    n = int(out.reshape(-1)[-1])
    d = mm.pixel_diagnostics(w.poses[1], 40, 30)
    assert n == len(d["s"]) > 0
    np.testing.assert_array_equal(out.reshape(-1)[:n * 10].reshape(n, 10)[:, 0], d["s"])
    out2 = np.zeros_like(out)
    inf.get_diagnostic_image_at_pose(w.poses[1], G.GVDBImage(w.depths[1]), out2)
    np.testing.assert_array_equal(out, out2)
    inf.get_diagnostic_image(1, out, 1)
    assert not out.any()
    cen = inf.get_occupied_bricks(0)
    vc = inf.get_voxel_coords([0, 1, 10 ** 9])
    np.testing.assert_array_equal(vc[:2, :3], cen[:2] - 4)
    np.testing.assert_array_equal(vc[:2, 3:], cen[:2] + 4)
    assert not vc[2].any()
