// GVDBMapLikelihoodEstimator.h -- likelihood of an externally supplied map
// (reference include/mrfmap/GVDBMapLikelihoodEstimator.h:46-134).
#pragma once
#include <memory>
#include <vector>

#include "GVDBImage.h"
#include "GVDBMRFMap.h"
#include "GVDBParams.h"

class GVDBMapLikelihoodEstimator {
 public:
  explicit GVDBMapLikelihoodEstimator(const gvdb_params_t& params, bool use_gl = false);

  gvdb_params_t params_;
  std::shared_ptr<GVDBMRFMap> map_;

  void add_camera(const float* pose, const std::shared_ptr<GVDBImage>& img);
  void set_pose(unsigned id, const float* pose);
  void activate_camera(int id) {}
  // points n x 3 in voxel units, occupancies n (load_map, .cpp:168-240)
  bool load_map(const float* points, const float* occupancies, int64_t n);
  float compute_likelihood(unsigned id);
  float get_likelihood_image(unsigned id, float* out_rowmajor);
  float get_likelihood_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                     float* out_rowmajor);
  float get_likelihood_image_at_pose_with_depth(const float* pose, const float* depth,
                                                float* out_rowmajor);
  // evaluation renders (src/GVDBMapLikelihoodEstimator.cpp:328-434)
  void get_accuracy_image(unsigned id, float* out_rowmajor);
  float get_accuracy_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                   float* out_rowmajor);
  float get_accuracy_image_at_pose_with_depth(const float* pose, const float* depth,
                                              float* out_rowmajor);
  float get_simple_accuracy_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img);
  float get_simple_accuracy_image_at_pose_with_depth(const float* pose, const float* depth,
                                                     float* out_rowmajor);
  void get_occ_thresh_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                    float* out_rowmajor, float occ_thresh);
  std::vector<float> get_occupied_bricks(int lev) { return map_->get_occupied_bricks(lev); }
  void get_alphas(float* out, int64_t rows, int64_t cols) { map_->get_alphas(out, rows, cols); }
  void set_selected_x_y(unsigned x, unsigned y) { sel_x_ = x; sel_y_ = y; }
  // the selected pixel's per-voxel ray records
  // (src/GVDBMapLikelihoodEstimator.cpp:436-500)
  void get_diagnostic_image(unsigned id, float* out_rowmajor);
  void get_diagnostic_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                    float* out_rowmajor);
  void set_acc_thresh(float t) { params_.acc_thresh = t; }

 private:
  std::vector<std::vector<float>> poses_;
  std::vector<std::shared_ptr<GVDBImage>> images_;
  unsigned sel_x_ = 0, sel_y_ = 0;
};
