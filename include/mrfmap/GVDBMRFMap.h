// GVDBMRFMap.h -- the map store (reference include/mrfmap/GVDBMRFMap.h),
// here the owner of one C-ABI map handle: a dense brick table and a pool of
// 8^3-voxel bricks in HBM.
#pragma once
#include <stdexcept>
#include <vector>

#include "../mrfmap_gb300.h"
#include "GVDBParams.h"

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

 private:
  mrf_map* map_ = nullptr;
};

// throws std::runtime_error carrying mrf_last_error() for non-OK statuses
void mrf_check(mrf_status st);
