// GVDBMapLikelihoodEstimator.h -- likelihood of an externally supplied map
// (reference include/mrfmap/GVDBMapLikelihoodEstimator.h:46-134).
#pragma once
#include <memory>
#include <vector>

#include "GVDBImage.h"
#include "GVDBMRFMap.h"
#include "GVDBParams.h"
#include "MatrixArgs.h"

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

  // The reference's signatures with Eigen arguments
  // (GVDBMapLikelihoodEstimator.h:97-117 there): any matrix type with
  // rows(), cols() and m(i, j).  load_map takes points n x 3 (voxel units)
  // and occupancies n x 1; output images have the camera's rows x cols.
  template <class P, class = mrf_shim::if_matrix<P>>
  void add_camera(const P& pose, const std::shared_ptr<GVDBImage>& img) {
    add_camera(mrf_shim::pose16(pose).data(), img);
  }
  template <class P, class = mrf_shim::if_matrix<P>>
  void set_pose(unsigned id, const P& pose) {
    set_pose(id, mrf_shim::pose16(pose).data());
  }
  template <class C, class V, class = mrf_shim::if_matrix<C>, class = mrf_shim::if_matrix<V>>
  bool load_map(const C& coords, const V& occupancies) {
    if (coords.cols() != 3 || (int64_t)occupancies.rows() * occupancies.cols() != (int64_t)coords.rows())
      throw std::runtime_error("load_map wants n x 3 points and n occupancies");
    const std::vector<float> c = mrf_shim::rowmajor(coords), o = mrf_shim::rowmajor(occupancies);
    return load_map(c.data(), o.data(), (int64_t)coords.rows());
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_likelihood_image(unsigned id, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const float s = get_likelihood_image(id, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_likelihood_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const float s = get_likelihood_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class D, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_matrix<D>,
            class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_likelihood_image_at_pose_with_depth(const P& pose, const D& depth, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const std::vector<float> d = mrf_shim::rowmajor(depth);
    const float s = get_likelihood_image_at_pose_with_depth(mrf_shim::pose16(pose).data(), d.data(), b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_accuracy_image(unsigned id, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    get_accuracy_image(id, b.data());
    mrf_shim::assign(out, b.data());
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_accuracy_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const float s = get_accuracy_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class D, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_matrix<D>,
            class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_accuracy_image_at_pose_with_depth(const P& pose, const D& depth, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const std::vector<float> d = mrf_shim::rowmajor(depth);
    const float s = get_accuracy_image_at_pose_with_depth(mrf_shim::pose16(pose).data(), d.data(), b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class = mrf_shim::if_matrix<P>>
  float get_simple_accuracy_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img) {
    return get_simple_accuracy_at_pose(mrf_shim::pose16(pose).data(), img);
  }
  template <class P, class D, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_matrix<D>,
            class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  float get_simple_accuracy_image_at_pose_with_depth(const P& pose, const D& depth, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    const std::vector<float> d = mrf_shim::rowmajor(depth);
    const float s =
        get_simple_accuracy_image_at_pose_with_depth(mrf_shim::pose16(pose).data(), d.data(), b.data());
    mrf_shim::assign(out, b.data());
    return s;
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_occ_thresh_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out,
                                    float occ_thresh) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    get_occ_thresh_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data(), occ_thresh);
    mrf_shim::assign(out, b.data());
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_alphas(O&& out) {
    map_->get_alphas(out);
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_diagnostic_image(unsigned id, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    get_diagnostic_image(id, b.data());
    mrf_shim::assign(out, b.data());
  }
  template <class P, class O, class = mrf_shim::if_matrix<P>, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_diagnostic_image_at_pose(const P& pose, const std::shared_ptr<GVDBImage>& img, O&& out) {
    std::vector<float> b = mrf_shim::image_scratch(out, params_.rows, params_.cols);
    get_diagnostic_image_at_pose(mrf_shim::pose16(pose).data(), img, b.data());
    mrf_shim::assign(out, b.data());
  }

 private:
  std::vector<std::vector<float>> poses_;
  std::vector<std::shared_ptr<GVDBImage>> images_;
  unsigned sel_x_ = 0, sel_y_ = 0;
};
