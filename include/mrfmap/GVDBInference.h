// GVDBInference.h -- the inference API of the reference
// (include/mrfmap/GVDBInference.h:36-102 in the MRFMap project) over the C
// ABI.  Poses are row-major 4x4 camera-to-world (metres); images row-major.
#pragma once
#include <memory>
#include <vector>

#include "GVDBImage.h"
#include "GVDBMRFMap.h"
#include "GVDBParams.h"

class GVDBInference {
 public:
  // use_gl is accepted and ignored (no graphics path); create_context is
  // accepted for signature compatibility: the map uses the current device.
  GVDBInference(bool create_context = true, bool use_gl = true);

  std::shared_ptr<GVDBMRFMap> map_;

  void add_camera(const float* pose, const std::shared_ptr<GVDBImage>& img);
  void add_camera_with_depth(const float* pose, const float* depth, int rows, int cols);
  void set_pose(unsigned id, const float* pose);
  void perform_inference();
  void perform_inference_dryrun();
  void perform_inference_ids(const std::vector<unsigned>& ids, bool dry_run = false);
  float compute_likelihood(unsigned id);
  float get_likelihood_image(unsigned id, float* out_rowmajor);
  float get_likelihood_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                     float* out_rowmajor);
  // evaluation renders (src/GVDBInference.cpp:242-247, 385-429)
  void get_expected_depth_image(unsigned id, float* out_rowmajor);
  float get_accuracy_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                   float* out_rowmajor);
  std::vector<float> get_occupied_bricks(int lev) { return map_->get_occupied_bricks(lev); }
  void get_alphas(float* out, int64_t rows, int64_t cols) { map_->get_alphas(out, rows, cols); }
  // debugging probes (src/GVDBInference.cpp:269-378): the selected pixel's
  // per-voxel ray records (mode 0; mode 1 records nothing under the
  // FULL_INFERENCE build), brick extents by slot (voxel units, n x 6)
  void get_diagnostic_image(unsigned id, float* out_rowmajor, unsigned mode = 0);
  void get_diagnostic_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                    float* out_rowmajor);
  std::vector<float> get_voxel_coords(const std::vector<uint64_t>& indices) const;
  // selected pixel of the diagnostics; the selected voxel is recorded only
  void set_selected_x_y(unsigned x, unsigned y) { sel_x_ = x; sel_y_ = y; }
  void set_selected_voxel(uint64_t id) { sel_vox_ = id; }
  size_t num_cameras() const { return n_cams_; }
  const std::vector<float>& get_cam_pose(unsigned id) const { return poses_.at(id); }
  // extensions: BP schedule / message flags of mrf_infer, and counters
  int infer_flags = 0;
  mrf_stats stats() const;

 private:
  size_t n_cams_ = 0;
  std::vector<std::vector<float>> poses_;
  unsigned sel_x_ = 0, sel_y_ = 0;
  uint64_t sel_vox_ = 0;
};
