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


@pytest.mark.skipif(not os.path.isdir("/root/reference/data"), reason="reference fixtures absent")
def test_reference_fixture_shapes():
    d = read_eigen_binary("/root/reference/data/depth_0.bin")
    P = read_eigen_binary("/root/reference/data/pose_0.bin")
    assert d.shape == (480, 640) and P.shape == (4, 4)
    assert np.isnan(d).sum() == 69120
