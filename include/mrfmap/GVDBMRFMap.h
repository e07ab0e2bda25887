// GVDBMRFMap.h -- the map store (reference include/mrfmap/GVDBMRFMap.h),
// here the owner of one C-ABI map handle: a dense brick table and a pool of
// 8^3-voxel bricks in HBM.
#pragma once
#include <stdexcept>
#include <vector>

#include "../mrfmap_gb300.h"
#include "GVDBParams.h"
#include "MatrixArgs.h"

class GVDBMRFMap {
 public:
  explicit GVDBMRFMap(const gvdb_params_t& params, int activation = MRF_ACT_ENDPOINT);
  ~GVDBMRFMap();
  GVDBMRFMap(const GVDBMRFMap&) = delete;
  GVDBMRFMap& operator=(const GVDBMRFMap&) = delete;

  mrf_map* handle() const { return map_; }
  int64_t num_bricks() const;
  // brick (lev 0) or node centres, n x 3, voxel units (GVDBMRFMap.cpp:137-152)
  std::vector<float> get_occupied_bricks(int lev) const;
  // [n_bricks x 512] beliefs, row-major (GVDBMRFMap.cpp:154-208); throws
  // std::runtime_error when rows/cols do not match
  void get_alphas(float* out, int64_t rows, int64_t cols) const;
  // [n_bricks x 16] int bitmask of belief >= threshold (GVDBMRFMap.cpp:210-263)
  void get_occupied_voxels_mask(int* out, int64_t rows, int64_t cols, float threshold) const;
  // the same with the reference's Eigen::Ref arguments (any writable matrix
  // type with rows(), cols() and m(i, j))
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_alphas(O&& out) const {
    std::vector<float> b((size_t)((int64_t)out.rows() * (int64_t)out.cols()));
    get_alphas(b.data(), (int64_t)out.rows(), (int64_t)out.cols());
    mrf_shim::assign(out, b.data());
  }
  template <class O, class = mrf_shim::if_out_matrix<mrf_shim::plain<O>>>
  void get_occupied_voxels_mask(O&& out, float threshold) const {
    std::vector<int> b((size_t)((int64_t)out.rows() * (int64_t)out.cols()));
    get_occupied_voxels_mask(b.data(), (int64_t)out.rows(), (int64_t)out.cols(), threshold);
    mrf_shim::assign(out, b.data());
  }

 private:
  mrf_map* map_ = nullptr;
};

// throws std::runtime_error carrying mrf_last_error() for non-OK statuses
void mrf_check(mrf_status st);
