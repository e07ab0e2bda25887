// GVDBShim.cpp -- the reference's C++ classes (GVDBInference, GVDBMRFMap,
// GVDBImage, GVDBMapLikelihoodEstimator, gvdb_params_t) implemented over the
// C ABI of libmrfmap_gb300.so.  Method names, argument meaning and error
// behaviour follow the reference; reference exits become exceptions.
#include <algorithm>
#include <cmath>
#include <fstream>
#include <map>
#include <sstream>
#include <stdexcept>
#include <string>

#include "mrfmap/GVDBImage.h"
#include "mrfmap/GVDBInference.h"
#include "mrfmap/GVDBMRFMap.h"
#include "mrfmap/GVDBMapLikelihoodEstimator.h"
#include "mrfmap/GVDBParams.h"

gvdb_params_t gvdb_params_;

void mrf_check(mrf_status st) {
  if (st != MRF_OK) throw std::runtime_error(std::string("mrfmap_gb300: ") + mrf_last_error());
}

// ---- YAML subset: "section:" then "  key: value" / "[a, b]" lists ----------
namespace {

std::string trim(const std::string& s) {
  size_t a = s.find_first_not_of(" \t\r"), b = s.find_last_not_of(" \t\r");
  return a == std::string::npos ? "" : s.substr(a, b - a + 1);
}

std::map<std::string, std::map<std::string, std::string>> parse_yaml(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("[gvdb_params] cannot read " + path);
  std::map<std::string, std::map<std::string, std::string>> out;
  std::string line, section, pending_key, pending;
  while (std::getline(f, line)) {
    auto h = line.find('#');
    if (h != std::string::npos) line = line.substr(0, h);
    if (trim(line).empty()) continue;
    if (!pending_key.empty()) {
      pending += " " + trim(line);
      if (pending.find(']') != std::string::npos) {
        out[section][pending_key] = pending;
        pending_key.clear();
      }
      continue;
    }
    if (line[0] != ' ' && line[0] != '\t') {
      section = trim(line);
      if (!section.empty() && section.back() == ':') section.pop_back();
      continue;
    }
    auto c = line.find(':');
    if (c == std::string::npos) continue;
    std::string key = trim(line.substr(0, c)), val = trim(line.substr(c + 1));
    if (!val.empty() && val[0] == '[' && val.find(']') == std::string::npos) {
      pending_key = key;
      pending = val;
    } else {
      out[section][key] = val;
    }
  }
  return out;
}

std::vector<float> as_list(const std::string& v) {
  std::string s = v;
  for (char& ch : s)
    if (ch == '[' || ch == ']' || ch == ',') ch = ' ';
  std::stringstream ss(s);
  std::vector<float> r;
  float x;
  while (ss >> x) r.push_back(x);
  return r;
}

bool as_bool(const std::string& v) {
  std::string s = v;
  std::transform(s.begin(), s.end(), s.begin(), ::tolower);
  return s == "true" || s == "1" || s == "yes";
}

std::vector<float> read_table(const std::string& path) {
  std::ifstream f(path);
  if (!f) throw std::runtime_error("[gvdb_params] cannot read " + path);
  std::stringstream ss;
  ss << f.rdbuf();
  return as_list(ss.str());
}

mrf_params to_mrf(const gvdb_params_t& p, int activation) {
  mrf_params m{};
  m.res = p.res;
  for (int a = 0; a < 3; ++a) m.dims[a] = p.dims[a];
  m.fx = p.K[0];
  m.fy = p.K[4];
  m.cx = p.K[2];
  m.cy = p.K[5];
  m.rows = p.rows;
  m.cols = p.cols;
  m.prior = p.prior;
  m.max_iters = (int)p.max_iters;
  m.lookup_n = p.lookup_n;
  m.sigma_lut = p.depth_sigma_lookup.data();
  m.bias_lut = p.depth_bias_lookup.data();
  m.occ_thresh = p.occ_thresh;
  m.acc_thresh = p.acc_thresh;
  m.activation = activation;
  return m;
}

}  // namespace

void gvdb_params_t::load_from_file(const std::string& file_path) {
  auto y = parse_yaml(file_path);
  if (!y.count("gvdb_params")) throw std::runtime_error("[gvdb_params] Could not read [gvdb_params]!");
  auto& g = y["gvdb_params"];
  if (g.count("rows")) rows = (int)std::stof(g["rows"]);
  if (g.count("cols")) cols = (int)std::stof(g["cols"]);
  if (g.count("dims")) {
    auto d = as_list(g["dims"]);
    for (int i = 0; i < 3 && i < (int)d.size(); ++i) dims[i] = d[i];
  }
  if (g.count("res")) res = std::stof(g["res"]);
  if (!g.count("use_polys"))
    throw std::runtime_error("[gvdb_params] Please configure use_polys in config file.");
  use_polys = as_bool(g["use_polys"]);
  int n_cells = n_tiles_u() * n_tiles_v();
  if (use_polys) {
    lookup_n = std::stoi(g["poly_degree"]);
    std::string base;
    auto pos = file_path.rfind('/');
    if (pos != std::string::npos) base = file_path.substr(0, pos + 1);
    auto strip = [](std::string s) {
      s = trim(s);
      if (s.size() >= 2 && (s[0] == '"' || s[0] == '\'')) s = s.substr(1, s.size() - 2);
      return s;
    };
    depth_sigma_lookup = read_table(base + strip(g["depth_sigma_lookup"]));
    depth_bias_lookup = read_table(base + strip(g["depth_bias_lookup"]));
    depth_sigma_lookup.resize((size_t)n_cells * lookup_n);
    depth_bias_lookup.resize((size_t)n_cells * lookup_n);
  } else if (g.count("const_sigmasq_poly")) {
    lookup_n = std::stoi(g["poly_degree"]);
    const_sigmasq_poly = as_list(g["const_sigmasq_poly"]);
    const_sigmasq_poly.resize(lookup_n);
    if (g.count("const_bias_poly")) {
      const_bias_poly = as_list(g["const_bias_poly"]);
      const_bias_poly.resize(lookup_n);
    }
    populate_lookup_tables();
  }
  if (g.count("prior")) prior = std::stof(g["prior"]);
  if (g.count("occ_thresh")) occ_thresh = std::stof(g["occ_thresh"]);
  if (g.count("acc_thresh")) acc_thresh = std::stof(g["acc_thresh"]);
  if (g.count("max_iters")) max_iters = (unsigned)std::stoi(g["max_iters"]);
  if (g.count("K")) {
    auto k = as_list(g["K"]);
    for (int i = 0; i < 9 && i < (int)k.size(); ++i) K[i] = k[i];
  }
  if (g.count("gvdb_map_config")) {
    auto c = as_list(g["gvdb_map_config"]);
    for (int i = 0; i < 5 && i < (int)c.size(); ++i) gvdb_map_config[i] = (int)c[i];
  }
  if (!use_polys && !g.count("const_sigmasq_poly")) populate_lookup_tables();
}

// ---- GVDBImage ---------------------------------------------------------------
GVDBImage::GVDBImage(const float* d, int rows, int cols) : GVDBImage(d, rows, cols, gvdb_params_) {}

GVDBImage::GVDBImage(const float* d, int rows, int cols, const gvdb_params_t& params)
    : depth_(d, d + (size_t)rows * cols), rows_(rows), cols_(cols), params_(params) {
  if (rows != params.rows || cols != params.cols)
    throw std::runtime_error("GVDBImage: image size does not match params rows x cols");
}

std::vector<float> GVDBImage::get_reproj_points() const {
  std::vector<float> pts;
  float fx = params_.K[0], cx = params_.K[2], cy = params_.K[5];
  for (int v = 0; v < rows_; ++v)
    for (int u = 0; u < cols_; ++u) {
      float d = depth_[(size_t)v * cols_ + u];
      if (!std::isfinite(d) || !(d > 0)) continue;
      float f = d / fx;
      pts.push_back(f * (u - cx));
      pts.push_back(f * (v - cy));
      pts.push_back(d);
    }
  return pts;
}

// ---- GVDBMRFMap ----------------------------------------------------------------
GVDBMRFMap::GVDBMRFMap(const gvdb_params_t& params, int activation) {
  mrf_params m = to_mrf(params, activation);
  mrf_check(mrf_create(&m, &map_));
}

GVDBMRFMap::~GVDBMRFMap() { mrf_destroy(map_); }

int64_t GVDBMRFMap::num_bricks() const {
  int64_t n = 0;
  mrf_check(mrf_num_bricks(map_, &n));
  return n;
}

std::vector<float> GVDBMRFMap::get_occupied_bricks(int lev) const {
  int64_t n = 0;
  mrf_check(mrf_num_nodes(map_, lev, &n));
  std::vector<float> c((size_t)n * 3);
  if (n) mrf_check(mrf_read_nodes(map_, lev, c.data(), n));
  return c;
}

void GVDBMRFMap::get_alphas(float* out, int64_t rows, int64_t cols) const {
  if (rows != num_bricks() || cols != 512)
    throw std::runtime_error("Dimensions for the alphas array are incorrect!");
  mrf_check(mrf_read_bricks(map_, nullptr, out, rows));
}

void GVDBMRFMap::get_occupied_voxels_mask(int* out, int64_t rows, int64_t cols, float thr) const {
  int64_t n = num_bricks();
  if (rows != n || cols != 16)
    throw std::runtime_error("Dimensions for the voxel mask array are incorrect!");
  std::vector<float> b((size_t)n * 512);
  if (n) mrf_check(mrf_read_bricks(map_, nullptr, b.data(), n));
  for (int64_t i = 0; i < n; ++i) {
    for (int w = 0; w < 16; ++w) out[i * 16 + w] = 0;
    for (int k = 0; k < 512; ++k)
      if (b[(size_t)i * 512 + k] >= thr) out[i * 16 + k / 32] |= (int)(1u << (k % 32));
  }
}

// ---- GVDBInference ---------------------------------------------------------------
GVDBInference::GVDBInference(bool, bool) : map_(std::make_shared<GVDBMRFMap>(gvdb_params_)) {}

void GVDBInference::add_camera(const float* pose, const std::shared_ptr<GVDBImage>& img) {
  int id = 0;
  mrf_check(mrf_add_view(map_->handle(), pose, img->depth().data(), &id));
  poses_.emplace_back(pose, pose + 16);
  n_cams_ = (size_t)id + 1;
}

void GVDBInference::add_camera_with_depth(const float* pose, const float* depth, int rows, int cols) {
  add_camera(pose, std::make_shared<GVDBImage>(depth, rows, cols));
}

void GVDBInference::set_pose(unsigned id, const float* pose) {
  mrf_check(mrf_set_pose(map_->handle(), (int)id, pose));
  poses_.at(id).assign(pose, pose + 16);
}

void GVDBInference::perform_inference() { perform_inference_ids({}, false); }
void GVDBInference::perform_inference_dryrun() { perform_inference_ids({}, true); }

void GVDBInference::perform_inference_ids(const std::vector<unsigned>& ids, bool) {
  // the reference's dry_run is unused with FULL_INFERENCE
  std::vector<int> v(ids.begin(), ids.end());
  mrf_check(mrf_infer(map_->handle(), ids.empty() ? nullptr : v.data(), (int)v.size(), 0, infer_flags));
}

float GVDBInference::compute_likelihood(unsigned id) { return get_likelihood_image(id, nullptr); }

float GVDBInference::get_likelihood_image(unsigned id, float* out) {
  float s = 0.0f;
  mrf_check(mrf_likelihood_view(map_->handle(), (int)id, out, &s));
  return s;
}

float GVDBInference::get_likelihood_image_at_pose(const float* pose,
                                                  const std::shared_ptr<GVDBImage>& img, float* out) {
  float s = 0.0f;
  mrf_check(mrf_likelihood(map_->handle(), pose, img->depth().data(), out, &s));
  return s;
}

void GVDBInference::get_expected_depth_image(unsigned id, float* out) {
  mrf_check(mrf_render_view(map_->handle(), MRF_RENDER_EXPECTED_DEPTH, (int)id, -1.0f, out, nullptr,
                            nullptr));
}

float GVDBInference::get_accuracy_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>& img,
                                                float* out) {
  float s = 0.0f;
  mrf_check(mrf_render(map_->handle(), MRF_RENDER_ACCURACY, pose, img->depth().data(), -1.0f, out, &s,
                       nullptr));
  return s;
}

void GVDBInference::get_diagnostic_image(unsigned id, float* out, unsigned mode) {
  const int64_t n = (int64_t)gvdb_params_.rows * gvdb_params_.cols;
  if (mode != 0) {  // the factor-debug mode records nothing under FULL_INFERENCE
    std::fill(out, out + n, 0.0f);
    return;
  }
  mrf_check(mrf_pixel_diagnostics(map_->handle(), poses_.at(id).data(), (int)sel_x_, (int)sel_y_, out, n));
}

void GVDBInference::get_diagnostic_image_at_pose(const float* pose, const std::shared_ptr<GVDBImage>&,
                                                 float* out) {
  const int64_t n = (int64_t)gvdb_params_.rows * gvdb_params_.cols;
  mrf_check(mrf_pixel_diagnostics(map_->handle(), pose, (int)sel_x_, (int)sel_y_, out, n));
}

std::vector<float> GVDBInference::get_voxel_coords(const std::vector<uint64_t>& indices) const {
  // brick slots -> world-frame (voxel units) min and max corners; unknown
  // slots give zeros, as the reference leaves rows of missing nodes at 0
  const int64_t n = map_->num_bricks();
  std::vector<float> c((size_t)n * 3);
  if (n) mrf_check(mrf_read_bricks(map_->handle(), c.data(), nullptr, n));
  std::vector<float> out(indices.size() * 6, 0.0f);
  for (size_t k = 0; k < indices.size(); ++k) {
    if (indices[k] >= (uint64_t)n) continue;
    for (int a = 0; a < 3; ++a) {
      out[k * 6 + a] = c[indices[k] * 3 + a] - 4.0f;
      out[k * 6 + 3 + a] = c[indices[k] * 3 + a] + 4.0f;
    }
  }
  return out;
}

mrf_stats GVDBInference::stats() const {
  mrf_stats s{};
  mrf_check(mrf_stats_get(map_->handle(), &s));
  return s;
}

// ---- GVDBMapLikelihoodEstimator ---------------------------------------------------
GVDBMapLikelihoodEstimator::GVDBMapLikelihoodEstimator(const gvdb_params_t& params, bool)
    : params_(params), map_(std::make_shared<GVDBMRFMap>(params)) {}

void GVDBMapLikelihoodEstimator::add_camera(const float* pose, const std::shared_ptr<GVDBImage>& img) {
  poses_.emplace_back(pose, pose + 16);
  images_.push_back(img);
}

void GVDBMapLikelihoodEstimator::set_pose(unsigned id, const float* pose) {
  poses_.at(id).assign(pose, pose + 16);
}

bool GVDBMapLikelihoodEstimator::load_map(const float* points, const float* occ, int64_t n) {
  mrf_check(mrf_load_map(map_->handle(), points, occ, n));
  return true;
}

float GVDBMapLikelihoodEstimator::compute_likelihood(unsigned id) {
  return get_likelihood_image(id, nullptr);
}

float GVDBMapLikelihoodEstimator::get_likelihood_image(unsigned id, float* out) {
  float s = 0.0f;
  mrf_check(mrf_likelihood(map_->handle(), poses_.at(id).data(), images_.at(id)->depth().data(), out, &s));
  return s;
}

float GVDBMapLikelihoodEstimator::get_likelihood_image_at_pose(
    const float* pose, const std::shared_ptr<GVDBImage>& img, float* out) {
  float s = 0.0f;
  mrf_check(mrf_likelihood(map_->handle(), pose, img->depth().data(), out, &s));
  return s;
}

float GVDBMapLikelihoodEstimator::get_likelihood_image_at_pose_with_depth(const float* pose,
                                                                        const float* depth, float* out) {
  float s = 0.0f;
  mrf_check(mrf_likelihood(map_->handle(), pose, depth, out, &s));
  return s;
}

void GVDBMapLikelihoodEstimator::get_accuracy_image(unsigned id, float* out) {
  get_accuracy_image_at_pose(poses_.at(id).data(), images_.at(id), out);
}

float GVDBMapLikelihoodEstimator::get_accuracy_image_at_pose(const float* pose,
                                                             const std::shared_ptr<GVDBImage>& img,
                                                             float* out) {
  return get_accuracy_image_at_pose_with_depth(pose, img->depth().data(), out);
}

float GVDBMapLikelihoodEstimator::get_accuracy_image_at_pose_with_depth(const float* pose,
                                                                        const float* depth, float* out) {
  float s = 0.0f;
  mrf_check(mrf_render(map_->handle(), MRF_RENDER_ACCURACY, pose, depth, -1.0f, out, &s, nullptr));
  return s;
}

float GVDBMapLikelihoodEstimator::get_simple_accuracy_at_pose(const float* pose,
                                                              const std::shared_ptr<GVDBImage>& img) {
  return get_simple_accuracy_image_at_pose_with_depth(pose, img->depth().data(), nullptr);
}

float GVDBMapLikelihoodEstimator::get_simple_accuracy_image_at_pose_with_depth(const float* pose,
                                                                               const float* depth,
                                                                               float* out) {
  float s = 0.0f;
  mrf_check(mrf_render(map_->handle(), MRF_RENDER_SIMPLE_ACCURACY, pose, depth, params_.acc_thresh, out,
                       &s, nullptr));
  return s;
}

void GVDBMapLikelihoodEstimator::get_occ_thresh_image_at_pose(const float* pose,
                                                              const std::shared_ptr<GVDBImage>& img,
                                                              float* out, float occ_thresh) {
  mrf_check(mrf_render(map_->handle(), MRF_RENDER_OCC_THRESH, pose, img->depth().data(), occ_thresh, out,
                       nullptr, nullptr));
}

void GVDBMapLikelihoodEstimator::get_diagnostic_image(unsigned id, float* out) {
  get_diagnostic_image_at_pose(poses_.at(id).data(), images_.at(id), out);
}

void GVDBMapLikelihoodEstimator::get_diagnostic_image_at_pose(const float* pose,
                                                              const std::shared_ptr<GVDBImage>&, float* out) {
  const int64_t n = (int64_t)params_.rows * params_.cols;
  mrf_check(mrf_pixel_diagnostics(map_->handle(), pose, (int)sel_x_, (int)sel_y_, out, n));
}
