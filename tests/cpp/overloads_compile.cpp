// Overload resolution of the shim's Eigen-style signatures (compiled to an
// object only: the calls resolve, nothing runs).  Each call is written the
// way a reference caller writes it (src/testMRFMapViewer.cpp:40-60,
// src/Viewer.cpp:44-61).
#include <memory>

#include "mock_matrix.h"
#include "mrfmap/GVDBInference.h"
#include "mrfmap/GVDBMapLikelihoodEstimator.h"

gvdb_params_t gvdb_params_;

void reference_style_calls(GVDBInference& inf, GVDBMapLikelihoodEstimator& est) {
  ColMajor<float> pose(4, 4), depth(480, 640), pts(10, 3), occ(10, 1);
  std::vector<float> buf(480 * 640), ab(512);
  RowRef<float> img{buf.data(), 480, 640, 640}, alphas{ab.data(), 1, 512, 512};
  std::vector<int> mb(16);
  RowRef<int> mask{mb.data(), 1, 16, 16};
  auto gimg = std::make_shared<GVDBImage>(depth);
  auto gimg2 = std::make_shared<GVDBImage>(depth, gvdb_params_);
  inf.add_camera(pose, gimg);
  inf.add_camera_with_depth(pose, depth);
  inf.set_pose(0, pose);
  float s = inf.get_likelihood_image(0, img);
  s += inf.get_likelihood_image_at_pose(pose, gimg, img);
  inf.get_expected_depth_image(0, img);
  s += inf.get_accuracy_image_at_pose(pose, gimg, img);
  inf.get_alphas(alphas);
  inf.get_diagnostic_image(0, img);
  inf.get_diagnostic_image(0, img, 1);
  inf.get_diagnostic_image_at_pose(pose, gimg2, img);
  inf.map_->get_occupied_voxels_mask(mask, 0.5f);
  // the pointer forms still resolve to themselves
  s += inf.get_likelihood_image(0, buf.data());
  s += inf.get_likelihood_image(0, nullptr);
  est.add_camera(pose, gimg);
  est.set_pose(0, pose);
  est.load_map(pts, occ);
  s += est.get_likelihood_image(0, img);
  s += est.get_likelihood_image_at_pose(pose, gimg, img);
  s += est.get_likelihood_image_at_pose_with_depth(pose, depth, img);
  est.get_accuracy_image(0, img);
  s += est.get_accuracy_image_at_pose(pose, gimg, img);
  s += est.get_accuracy_image_at_pose_with_depth(pose, depth, img);
  s += est.get_simple_accuracy_at_pose(pose, gimg);
  s += est.get_simple_accuracy_image_at_pose_with_depth(pose, depth, img);
  est.get_occ_thresh_image_at_pose(pose, gimg, img, 0.5f);
  est.get_alphas(alphas);
  est.get_diagnostic_image(0, img);
  est.get_diagnostic_image_at_pose(pose, gimg, img);
  (void)s;
}
