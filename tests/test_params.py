"""Host-side parameter handling (mirror of gvdb_params_t)."""
import math
import os

import numpy as np
import pytest

from mrfmap_gb300.params import MapParams, parse_flat_yaml, read_eigen_binary

YAML = """
viewer_params_nodes:
  cam_in_body: [ 0., 0. , 1., 0.,
                -1.,  0., 0., 0.,
                0.,  -1., 0., 0.,
                0.,  0.,  0.,  1.]
  camera_topic: '/camera/depth/image'

gvdb_params:
  K: [381.5, 0., 319.5, 0., 381.5, 239.5, 0., 0., 1.]
  res: 0.02                # Map resolution in m
  prior: 0.1
  dims: [4.0, 4.0, 3.0]
  occ_thresh: 0.5
  acc_thresh: 0.1
  max_iters: 3
  gvdb_map_config: [3, 3, 3, 3, 3]
  rows: 480
  cols: 640
  use_polys: False
  poly_degree: 3
  depth_sigma_lookup: ""
  const_sigmasq_poly: [0.05, 0, 0]
"""


def test_yaml_subset():
    y = parse_flat_yaml(YAML)
    assert y["gvdb_params"]["res"] == 0.02
    assert y["gvdb_params"]["use_polys"] is False
    assert len(y["viewer_params_nodes"]["cam_in_body"]) == 16
    assert y["gvdb_params"]["K"][2] == 319.5


def test_load_from_file(tmp_path):
    f = tmp_path / "cfg.yaml"
    f.write_text(YAML)
    p = MapParams().load_from_file(str(f))
    assert (p.rows, p.cols, p.res, p.prior, p.max_iters) == (480, 640, 0.02, 0.1, 3)
    assert (p.fx, p.cx, p.fy, p.cy) == (381.5, 319.5, 381.5, 239.5)
    assert p.dims == (4.0, 4.0, 3.0)
    # one polynomial per 20x20 tile: 32 x 24 tiles x 3 coefficients
    assert p.sigma_lut.shape == (32 * 24 * 3,)
    np.testing.assert_array_equal(p.sigma_lut.reshape(-1, 3), np.tile(np.float32([0.05, 0, 0]), (768, 1)))
    np.testing.assert_array_equal(p.bias_lut, 0)
    p.check()


def test_missing_use_polys_is_an_error(tmp_path):
    f = tmp_path / "cfg.yaml"
    f.write_text(YAML.replace("  use_polys: False\n", ""))
    with pytest.raises(ValueError):
        MapParams().load_from_file(str(f))


def test_defaults_match_reference():
    p = MapParams()
    assert p.res == 0.01 and p.prior == 0.01 and p.max_iters == 1
    assert p.fx == pytest.approx((1 / 2.0) / math.tan(0.005))


def test_eigen_binary_reader(tmp_path):
    a = np.arange(12, dtype=np.float32).reshape(3, 4)
    f = tmp_path / "m.bin"
    with open(f, "wb") as fh:
        fh.write(np.array([3, 4], np.int64).tobytes())
        fh.write(a.T.copy().tobytes())  # column-major
    np.testing.assert_array_equal(read_eigen_binary(str(f)), a)


REFERENCE = os.environ.get("MRFMAP_REFERENCE_DIR")
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "coffin_world.npz")


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(os.path.join(REFERENCE or "", "data")),
                    reason="MRFMAP_REFERENCE_DIR unset or without data/")
def test_reference_fixture_shapes():
    d = read_eigen_binary(os.path.join(REFERENCE, "data", "depth_0.bin"))
    P = read_eigen_binary(os.path.join(REFERENCE, "data", "pose_0.bin"))
    assert d.shape == (480, 640) and P.shape == (4, 4)
    assert np.isnan(d).sum() == 69120


@pytest.mark.skipif(not REFERENCE or not os.path.isdir(os.path.join(REFERENCE or "", "data")),
                    reason="MRFMAP_REFERENCE_DIR unset or without data/")
def test_golden_fixture_is_the_reference_data():
    """tests/golden/coffin_world.npz holds the reference's frames unchanged
    (row-major) and its body poses times cam_in_body."""
    g = np.load(GOLDEN)
    for k in (0, 7, 12):
        d = read_eigen_binary(os.path.join(REFERENCE, "data", f"depth_{k}.bin"))
        np.testing.assert_array_equal(g["depth"][k].view(np.uint32), d.view(np.uint32))
        body = read_eigen_binary(os.path.join(REFERENCE, "data", f"pose_{k}.bin")).astype(np.float64)
        np.testing.assert_allclose(g["pose"][k], body @ _cam_in_body(),
                                   rtol=0, atol=1e-6)


def _cam_in_body():
    # config/coffin_world_640.yaml viewer_params_nodes.cam_in_body, row by row
    return np.array([[0, 0, 1, 0], [-1, 0, 0, 0], [0, -1, 0, 0], [0, 0, 0, 1]], np.float64)


def test_golden_fixture_loads_as_reference_config(tmp_path):
    """The committed fixture's config parses to the reference's map and
    sensor parameters (config/coffin_world_640.yaml:16-34)."""
    g = np.load(GOLDEN)
    f = tmp_path / "coffin_world_640.yaml"
    f.write_text(str(g["yaml"]))
    p = MapParams().load_from_file(str(f))
    assert (p.rows, p.cols, p.res, p.dims, p.max_iters) == (480, 640, 0.02, (4.0, 4.0, 3.0), 3)
    assert (p.fx, p.fy, p.cx, p.cy) == (381.36115025, 381.36115025, 319.5, 239.5)
    assert p.use_polys is False and p.lookup_n == 3 and p.prior == pytest.approx(0.1)
    np.testing.assert_array_equal(p.sigma_lut[:3], np.float32([0.05, 0.0, 0.0]))
    assert g["depth"].shape == (13, 480, 640) and g["pose"].shape == (13, 4, 4)
    assert np.isnan(g["depth"]).sum() == 13 * 69120
    # camera z axis of frame 0 points from (3, 0, 2) m down towards the volume
    np.testing.assert_allclose(g["pose"][0][:3, 3], [3.0, 0.0, 2.0], atol=1e-6)
    assert g["pose"][0][2, 2] < 0
