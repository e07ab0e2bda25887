// GVDBInference.h -- the inference API of the reference
// (include/mrfmap/GVDBInference.h:36-102 in the MRFMap project) over the C
// ABI.  Poses are row-major 4x4 camera-to-world (metres); images row-major.
#pragma once
#include <memory>
#include <vector>

#include "GVDBImage.h"
#include "GVDBMRFMap.h"
#include "GVDBParams.h"
#include "MatrixArgs.h"

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

  // The reference's signatures with Eigen arguments (GVDBInference.h:87-102
  // there): any matrix type with rows(), cols() and m(i, j) -- column-major
  // Eigen::MatrixXf poses and images in, Eigen::Ref<MRow> images out.
  // Output images have the camera's rows x cols (std::runtime_error else).
  template <class P, class = mrf_shim::if_matrix<P>>
  void add_camera(const P& pose, const std::shared_ptr<GVDBImage>& img) {
    add_camera(mrf_shim::pose16(pose).data(), img);
  }
  template <class P, class D, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_matrix<D>>
  void add_camera_with_depth(const P& pose, const D& depth) {
    const std::vector<float> d = mrf_shim::rowmajor(depth);
    add_camera_with_depth(mrf_shim::pose16(pose).data(), d.data(), (int)depth.rows(), (int)depth.cols());
  }
  template <class P, class = mrf_shim::if_matrix<P>>
  void set_pose(unsigned id, const P& pose) {
    set_pose(id, mrf_shim::pose16(pose).data());
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_likelihood_image(unsigned id, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    const float s = get_likelihood_image(id, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_likelihood_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    const float s = get_likelihood_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_expected_depth_image(unsigned id, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    get_expected_depth_image(id, b.data());
    mrf_shim::assign(out, b.data());
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_accuracy_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    const float s = get_accuracy_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_alphas(O&& out) {
    map_->get_alphas(out);
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_diagnostic_image(unsigned id, O&& out, unsigned mode = 0) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    get_diagnostic_image(id, b.data(), mode);
    mrf_shim::assign(out, b.data());
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_diagnostic_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, gvdb_params_.rows, gvdb_params_.cols);
    get_diagnostic_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
  }

 private:
  size_t n_cams_ = 0;
  std::vector<std::vector<float>> poses_;
  unsigned sel_x_ = 0, sel_y_ = 0;
  uint64_t sel_vox_ = 0;
};
