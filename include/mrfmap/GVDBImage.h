// GVDBImage.h -- a depth image handed to the map (reference:
// include/mrfmap/GVDBImage.h).  Holds the row-major depth (metres, row 0 at
// the top); upload and clean-up (NaN -> -1) happen when a camera is added.
#pragma once
#include <memory>
#include <vector>

#include "GVDBParams.h"
#include "MatrixArgs.h"

class GVDBImage {
 public:
  GVDBImage(const float* depth_rowmajor, int rows, int cols);
  GVDBImage(const float* depth_rowmajor, int rows, int cols, const gvdb_params_t& params);
  // the reference's GVDBImage(const Eigen::MatrixXf&[, params]): any matrix
  // type with rows(), cols() and m(i, j)
  template <class M, class = mrf_shim::if_matrix<M>>
  GVDBImage(const M& depth)
      : GVDBImage(mrf_shim::rowmajor(depth).data(), (int)depth.rows(), (int)depth.cols()) {}
  template <class M, class = mrf_shim::if_matrix<M>>
  GVDBImage(const M& depth, const gvdb_params_t& params)
      : GVDBImage(mrf_shim::rowmajor(depth).data(), (int)depth.rows(), (int)depth.cols(), params) {}
  const std::vector<float>& depth() const { return depth_; }
  int rows() const { return rows_; }
  int cols() const { return cols_; }
  // back-projected valid pixels (n x 3, camera frame), GVDBImage.cpp:48-60
  std::vector<float> get_reproj_points() const;

 private:
  std::vector<float> depth_;
  int rows_, cols_;
  gvdb_params_t params_;
};
