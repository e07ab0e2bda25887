"""The GVDBPyModules mirror exposes the reference module's classes and
methods for the path (src/GVDBPyModules.cpp:42-135): import and attribute
checks only, no device calls, so this runs without a GPU.  Left out, as
the design records: PangolinViewer (graphics), GVDBOctomapWrapper (OctoMap
absent) and GVDBMapLikelihoodEstimator.get_rendered_image[_at_pose]
(GVDB's own display shading)."""
import glob
import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

SURFACE = {
    "gvdb_params": ["prior", "res", "dims", "const_sigmasq_poly", "occ_thresh", "max_iters", "rows", "cols",
                    "K", "use_polys", "lookup_n", "load_from_file", "set_from_python"],
    "GVDBInference": ["add_camera", "add_camera_with_depth", "perform_inference", "perform_inference_dryrun",
                      "set_pose", "get_likelihood_image", "get_expected_depth_image", "compute_likelihood",
                      "set_selected_x_y", "set_selected_voxel", "set_owned_context", "get_voxel_coords",
                      "get_diagnostic_image", "get_diagnostic_image_at_pose", "get_occupied_bricks",
                      "get_indices_and_alphas", "get_accuracy_image_at_pose", "get_likelihood_image_at_pose"],
    "GVDBMapLikelihoodEstimator": [
        "add_camera", "activate_camera", "load_map", "compute_likelihood", "set_selected_x_y",
        "set_acc_thresh", "get_diagnostic_image", "get_diagnostic_image_at_pose", "get_accuracy_image",
        "get_accuracy_image_at_pose", "get_accuracy_image_at_pose_with_depth", "get_simple_accuracy_at_pose",
        "get_simple_accuracy_image_at_pose_with_depth", "get_likelihood_image_at_pose",
        "get_likelihood_image_at_pose_with_depth", "get_occ_thresh_image_at_pose", "get_occupied_bricks",
        "get_indices_and_alphas", "get_likelihood_image"],
    "KeyframeSelector": ["compute_distance", "is_keyframe"],
    "GVDBImage": [],
}


@pytest.fixture(scope="module")
def pymod():
    from mrfmap_gb300 import _build
    libdir = os.path.join(ROOT, "mrfmap_gb300", "_lib")
    if not glob.glob(os.path.join(libdir, "GVDBPyModules*.so")):
        _build.build_pymodule()
    if libdir not in sys.path:
        sys.path.insert(0, libdir)
    import GVDBPyModules
    return GVDBPyModules


@pytest.mark.parametrize("cls", sorted(SURFACE))
def test_reference_surface(pymod, cls):
    assert hasattr(pymod, cls), cls
    c = getattr(pymod, cls)
    for name in SURFACE[cls]:
        assert hasattr(c, name), f"{cls}.{name}"
