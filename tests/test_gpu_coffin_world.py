"""The reference's own input fixture through both sides.

Frames, poses and config of the reference's viewer test
(``config/coffin_world_640.yaml``, ``data/depth_*.bin``, ``data/pose_*.bin``,
loaded as in ``src/testMRFMapViewer.cpp:18-67``), repacked by
``tests/golden/make_coffin_world.py``: 640x480 with the principal point at
(319.5, 239.5), 2 cm voxels in a 4x4x3 m volume the cameras look into from
outside, a constant sensor polynomial (``use_polys: False``), 69,120 NaN
pixels per frame, endpoint activation (the reference's policy) and the
viewer's loop -- for every keyframe ``add_camera`` then
``perform_inference`` with ``max_iters`` = 3 (``src/Viewer.cpp:44-61``),
which zeroes every camera's messages but not the total log-odds.

The CUDA path (through the C ABI) is compared with the FP64 oracle: brick
sets and incidence lists bit-exact, beliefs within 1e-3 with >= 99.9 %
class agreement along the loop, likelihood images within 1e-3 on the same
belief field."""
import os

import numpy as np
import pytest

from mrfmap_gb300 import lib as L
from mrfmap_gb300.params import MapParams
from oracle import oracle as O

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURE = os.path.join(HERE, "golden", "coffin_world.npz")
BELIEF_TOL = 1e-3
AGREE_MIN = 0.999
LIKE_TOL = 1e-3


@pytest.fixture(scope="module")
def coffin(native_lib, oracle_lib, tmp_path_factory):
    d = np.load(FIXTURE)
    cfg = tmp_path_factory.mktemp("coffin") / "coffin_world_640.yaml"
    cfg.write_text(str(d["yaml"]))
    p = MapParams().load_from_file(str(cfg))
    kf = np.flatnonzero(d["keyframe"])
    return p, d["pose"], d["depth"], kf


def _compare(gb, ob):
    gb = gb.astype(np.float64)
    touched = (gb > 0) | (ob > 0)
    return float(np.abs(gb - ob).max()), float(((gb > 0.5) == (ob > 0.5))[touched].mean())


def test_fixture_is_the_reference_config(coffin):
    p, pose, depth, kf = coffin
    assert (p.rows, p.cols) == (480, 640) and (p.cx, p.cy) == (319.5, 239.5)
    assert p.res == 0.02 and p.dims == (4.0, 4.0, 3.0) and p.max_iters == 3
    assert not p.use_polys and p.const_sigmasq_poly[0] == 0.05
    assert depth.shape == (13, 480, 640) and np.isnan(depth).sum(axis=(1, 2)).tolist() == [69120] * 13
    assert kf.tolist() == list(range(12))


def test_viewer_loop_matches_oracle(coffin):
    p, pose, depth, kf = coffin
    gm = L.MRFMap(p, activation=L.ACT_ENDPOINT)
    om = O.OracleMap(p, threads=os.cpu_count() or 1)
    errs = []
    for n, k in enumerate(kf):
        gm.add_view(pose[k], depth[k])
        om.add_view(pose[k], depth[k], O.ACT_ENDPOINT)
        gm.infer()          # perform_inference(): all cameras zeroed, max_iters iterations
        om.infer()
        assert gm.num_bricks == om.num_bricks
        if n in (0, len(kf) // 2, len(kf) - 1):
            emax, agree = _compare(gm.beliefs(), om.beliefs())
            errs.append(emax)
            assert emax <= BELIEF_TOL, f"keyframe {k}: max belief error {emax}"
            assert agree >= AGREE_MIN, f"keyframe {k}: class agreement {agree}"
    np.testing.assert_array_equal(gm.brick_coords(), om.brick_coords())
    # incidence lists of the first, a middle and the last view, bit for bit
    H, W = p.rows, p.cols
    for v in (0, len(kf) // 2, len(kf) - 1):
        meta, vox, ln, mu = gm.view_incidences(v)
        t = om.view_trace(v)
        ometa = np.zeros((H * W, 5), np.int32)
        ometa[t["pix"]] = t["meta"]
        np.testing.assert_array_equal(meta, ometa)
        np.testing.assert_array_equal(vox.astype(np.int64), t["vox"].astype(np.int64))
        np.testing.assert_array_equal(ln.view(np.uint32), t["len"].view(np.uint32))
        np.testing.assert_array_equal(mu == 0, t["mu"] == 0)
    # likelihood of two frames on the same belief field (a keyframe and the
    # frame the viewer test never loads)
    om.set_beliefs(gm.beliefs())
    for k in (kf[3], 12):
        gs, gimg = gm.likelihood(pose[k], depth[k])
        os_, oimg = om.likelihood(pose[k], depth[k])
        np.testing.assert_allclose(gimg, oimg, atol=LIKE_TOL, rtol=0)
        assert np.all(gimg[np.isnan(depth[k])] == 0)
    gm.close()
    om.close()
