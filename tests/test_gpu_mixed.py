"""Views of mixed resolution in one map (the batched uneven workload): each
view has its own camera (mrf_add_view_camera); the sensor tables are looked
up at pixel positions scaled into the params' image.  Parity against the
oracle's per-view cameras, as for single-camera maps."""
import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300 import synthetic
from oracle import oracle as O

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def mixed(native_lib, oracle_lib):
    w = synthetic.mixed_room(2, n_frames=6)
    gm = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    om = O.OracleMap(w.params, threads=8)
    for P, D, (fx, fy, cx, cy) in zip(w.poses, w.depths, w.cams):
        gm.add_view_camera(P, D, fx, fy, cx, cy)
        om.add_view_camera(P, D, D.shape[0], D.shape[1], fx, fy, cx, cy, O.ACT_FULL_RAY)
    return w, gm, om


def test_views_keep_their_cameras(mixed):
    w, gm, _ = mixed
    for v, (D, cam) in enumerate(zip(w.depths, w.cams)):
        rows, cols, k = gm.view_camera(v)
        assert (rows, cols) == D.shape
        np.testing.assert_allclose(k, cam, rtol=1e-6)


def test_bricks_and_incidences_bit_exact(mixed):
    w, gm, om = mixed
    assert gm.num_bricks == om.num_bricks
    np.testing.assert_array_equal(gm.brick_coords(), om.brick_coords())
    for v, D in enumerate(w.depths):
        meta, vox, ln, mu = gm.view_incidences(v)
        t = om.view_trace(v)
        ometa = np.zeros((D.size, 5), np.int32)
        ometa[t["pix"]] = t["meta"]
        np.testing.assert_array_equal(meta, ometa)
        np.testing.assert_array_equal(vox.astype(np.int64), t["vox"].astype(np.int64))
        np.testing.assert_array_equal(ln.view(np.uint32), t["len"].view(np.uint32))
        np.testing.assert_array_equal(mu == 0, t["mu"] == 0)


@pytest.mark.parametrize("flags", [0, L.JACOBI], ids=["gauss-seidel", "jacobi"])
def test_beliefs_match_oracle(mixed, flags):
    w, gm, om = mixed
    gm.reset_state()
    gm.infer(iters=8, flags=flags)
    om2 = O.OracleMap(w.params, threads=8)
    for P, D, (fx, fy, cx, cy) in zip(w.poses, w.depths, w.cams):
        om2.add_view_camera(P, D, D.shape[0], D.shape[1], fx, fy, cx, cy, O.ACT_FULL_RAY)
    om2.infer(iters=8, flags=O.JACOBI if flags else 0)
    gb, ob = gm.beliefs().astype(np.float64), om2.beliefs()
    touched = (gb > 0) | (ob > 0)
    assert np.abs(gb - ob).max() <= 1e-3
    assert ((gb > 0.5) == (ob > 0.5))[touched].mean() >= 0.999


def test_view_outputs_have_the_view_size(mixed):
    w, gm, om = mixed
    gm.reset_state()
    gm.infer(iters=4)
    for v, D in enumerate(w.depths[:3]):
        s, img = gm.likelihood_view(v)
        assert img.shape == D.shape and np.isfinite(s)
        img2, _, cnt = gm.render_view(L.RENDER_ACCURACY, v)
        assert img2.shape == D.shape and cnt.sum() == D.size
    # the largest views use the params' camera: same as the likelihood at pose
    v = 2
    s, img = gm.likelihood_view(v)
    s2, img2 = gm.likelihood(w.poses[v], w.depths[v])
    np.testing.assert_array_equal(img, img2)


def test_own_camera_equals_params_camera(native_lib):
    """A view added with the params' own camera is the same view."""
    w = synthetic.small_room(0, n_frames=2)
    a = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    b = L.MRFMap(w.params, activation=L.ACT_FULL_RAY)
    p = w.params
    for P, D in zip(w.poses, w.depths):
        a.add_view(P, D)
        b.add_view_camera(P, D, p.fx, p.fy, p.cx, p.cy)
    a.infer(iters=3)
    b.infer(iters=3)
    np.testing.assert_array_equal(a.beliefs(), b.beliefs())
    with pytest.raises(L.MrfError):
        b.add_view_camera(w.poses[0], w.depths[0], -1.0, p.fy, p.cx, p.cy)
