// GVDBParams.h -- host parameters of a map, mirroring the reference's
// gvdb_params_t (include/mrfmap/GVDBParams.h:11-104 in the MRFMap project):
// same field names, defaults, per-20x20-tile sensor polynomial tables and
// YAML keys.  Eigen types become plain arrays: dims[3], K[9] (row-major).
#pragma once
#include <array>
#include <cmath>
#include <string>
#include <vector>

#define MRF_LOOKUP_NUM 3096
#define MRF_LOOKUP_PX 20

struct gvdb_params_t {
  float hfov = 0.01f;
  float res = 0.01f;
  std::vector<float> const_sigmasq_poly{0.015f, 0.0f, 0.0f};
  std::vector<float> const_bias_poly{0.0f, 0.0f, 0.0f};
  float occ_thresh = 0.1f, acc_thresh = 0.5f;
  float prior = 0.01f;
  unsigned max_iters = 1;
  std::array<float, 3> dims{1.0f, 1.0f, 1.0f};
  int rows = 1, cols = 1;
  std::array<float, 9> K{};  // row-major 3x3
  bool use_polys = false;
  int lookup_n = 3;
  std::vector<float> depth_sigma_lookup, depth_bias_lookup;
  std::array<int, 5> gvdb_map_config{1, 3, 3, 3, 3};

  gvdb_params_t() {
    K = {0, 0, 0, 0, 0, 0, 0, 0, 1};
    K[0] = K[4] = (cols / 2.0f) / std::tan(hfov / 2.0f);
    K[2] = cols * 0.5f;
    K[5] = rows * 0.5f;
    const_sigmasq_poly = {1.5f * res, 0.0f, 0.0f};
    populate_lookup_tables();
  }

  int n_tiles_u() const { return (cols + MRF_LOOKUP_PX - 1) / MRF_LOOKUP_PX; }
  int n_tiles_v() const { return (rows + MRF_LOOKUP_PX - 1) / MRF_LOOKUP_PX; }

  // GVDBParams.h:93-104: replicate the constant polynomials per tile
  void populate_lookup_tables() {
    int n = n_tiles_u() * n_tiles_v();
    depth_sigma_lookup.assign((size_t)n * lookup_n, 0.0f);
    depth_bias_lookup.assign((size_t)n * lookup_n, 0.0f);
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < lookup_n; ++j) {
        depth_sigma_lookup[i * lookup_n + j] = j < (int)const_sigmasq_poly.size() ? const_sigmasq_poly[j] : 0.0f;
        depth_bias_lookup[i * lookup_n + j] = j < (int)const_bias_poly.size() ? const_bias_poly[j] : 0.0f;
      }
  }

  // GVDBParams.h:106-214: the gvdb_params block of a YAML config.  Throws
  // std::runtime_error where the reference prints and exits.
  void load_from_file(const std::string& file_path);
};

// process-wide parameters used by GVDBInference/GVDBImage
// (src/GVDBPyModules.cpp:23 in the reference)
extern gvdb_params_t gvdb_params_;
