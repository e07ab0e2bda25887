// GVDBPyModules.cpp -- the reference's Python module (src/GVDBPyModules.cpp:31-134
// in the MRFMap project): gvdb_params, GVDBImage, GVDBInference and
// GVDBMapLikelihoodEstimator with the same method names.  Matrices are numpy
// arrays: poses 4x4, depth rows x cols, outputs are caller-allocated float32
// C-contiguous arrays filled in place (as Eigen::Ref<MRow> arguments are).
// Viewer, OctoMap and keyframe-selector bindings are not part of this module.
#include <pybind11/numpy.h>
#include <pybind11/pybind11.h>
#include <pybind11/stl.h>

#include <stdexcept>
#include <string>

#include "mrfmap/GVDBImage.h"
#include "mrfmap/GVDBInference.h"
#include "mrfmap/GVDBMapLikelihoodEstimator.h"
#include "mrfmap/KeyframeSelector.h"
#include "mrfmap/GVDBParams.h"

namespace py = pybind11;
using farr = py::array_t<float, py::array::c_style | py::array::forcecast>;

namespace {

std::vector<float> pose16(const farr& p) {
  if (p.ndim() != 2 || p.shape(0) != 4 || p.shape(1) != 4) throw std::invalid_argument("pose must be 4x4");
  return std::vector<float>(p.data(), p.data() + 16);
}

float* out_buffer(py::array& out, int64_t rows, int64_t cols, const char* what) {
  if (!py::isinstance<py::array_t<float>>(out) || !(out.flags() & py::array::c_style) || !out.writeable())
    throw py::type_error(std::string(what) + " must be a writeable C-contiguous float32 array");
  if (out.ndim() != 2 || out.shape(0) != rows || out.shape(1) != cols)
    throw std::runtime_error(std::string("Dimensions for the ") + what + " array are incorrect!");
  return static_cast<float*>(out.mutable_data());
}

void check_depth(const farr& depth, const gvdb_params_t& p) {
  if (depth.ndim() != 2 || depth.shape(0) != p.rows || depth.shape(1) != p.cols)
    throw std::invalid_argument("depth image size does not match params");
}

std::shared_ptr<GVDBImage> make_image(const farr& d, const gvdb_params_t& p) {
  if (d.ndim() != 2) throw std::invalid_argument("depth image must be 2-D");
  return std::make_shared<GVDBImage>(d.data(), (int)d.shape(0), (int)d.shape(1), p);
}

py::array_t<float> bricks_array(const std::vector<float>& c) {
  py::array_t<float> a({(py::ssize_t)(c.size() / 3), (py::ssize_t)3});
  std::copy(c.begin(), c.end(), a.mutable_data());
  return a;
}

}  // namespace

PYBIND11_MODULE(GVDBPyModules, m) {
  m.doc() = "Occupancy inference (MRFMap forward-ray-sensor-model BP) on GB300";

  py::class_<gvdb_params_t>(m, "gvdb_params")
      .def(py::init<>())
      .def_readwrite("prior", &gvdb_params_t::prior)
      .def_readwrite("res", &gvdb_params_t::res)
      .def_property(
          "dims", [](const gvdb_params_t& p) { return std::vector<float>(p.dims.begin(), p.dims.end()); },
          [](gvdb_params_t& p, std::vector<float> v) {
            if (v.size() != 3) throw std::invalid_argument("dims needs 3 values");
            for (int i = 0; i < 3; ++i) p.dims[i] = v[i];
          })
      .def_readwrite("const_sigmasq_poly", &gvdb_params_t::const_sigmasq_poly)
      .def_readwrite("const_bias_poly", &gvdb_params_t::const_bias_poly)
      .def_readwrite("occ_thresh", &gvdb_params_t::occ_thresh)
      .def_readwrite("acc_thresh", &gvdb_params_t::acc_thresh)
      .def_readwrite("max_iters", &gvdb_params_t::max_iters)
      .def_readwrite("rows", &gvdb_params_t::rows)
      .def_readwrite("cols", &gvdb_params_t::cols)
      .def_property(
          "K",
          [](const gvdb_params_t& p) {
            py::array_t<float> a({3, 3});
            std::copy(p.K.begin(), p.K.end(), a.mutable_data());
            return a;
          },
          [](gvdb_params_t& p, farr k) {
            if (k.size() != 9) throw std::invalid_argument("K must be 3x3");
            std::copy(k.data(), k.data() + 9, p.K.begin());
          })
      .def_readwrite("use_polys", &gvdb_params_t::use_polys)
      .def_readwrite("lookup_n", &gvdb_params_t::lookup_n)
      .def_readwrite("depth_sigma_lookup", &gvdb_params_t::depth_sigma_lookup)
      .def_readwrite("depth_bias_lookup", &gvdb_params_t::depth_bias_lookup)
      .def("populate_lookup_tables", &gvdb_params_t::populate_lookup_tables)
      .def("load_from_file", &gvdb_params_t::load_from_file)
      .def("set_from_python", [](gvdb_params_t& self) { gvdb_params_ = self; });

  py::class_<GVDBImage, std::shared_ptr<GVDBImage>>(m, "GVDBImage")
      .def(py::init([](farr d) { return make_image(d, gvdb_params_); }))
      .def(py::init([](farr d, const gvdb_params_t& p) { return make_image(d, p); }));

  py::class_<GVDBInference, std::shared_ptr<GVDBInference>>(m, "GVDBInference")
      .def(py::init<bool, bool>(), py::arg("create_context") = true, py::arg("use_gl") = true)
      .def("add_camera", [](GVDBInference& s, farr pose, std::shared_ptr<GVDBImage> img) {
        s.add_camera(pose16(pose).data(), img);
      })
      .def("add_camera_with_depth", [](GVDBInference& s, farr pose, farr depth) {
        s.add_camera(pose16(pose).data(), make_image(depth, gvdb_params_));
      })
      .def("perform_inference", &GVDBInference::perform_inference)
      .def("perform_inference_dryrun", &GVDBInference::perform_inference_dryrun)
      .def("perform_inference_ids", &GVDBInference::perform_inference_ids, py::arg("ids"),
           py::arg("dry_run") = false)
      .def("set_pose", [](GVDBInference& s, unsigned id, farr pose) { s.set_pose(id, pose16(pose).data()); })
      .def("get_likelihood_image", [](GVDBInference& s, unsigned id, py::array out) {
        return s.get_likelihood_image(id, out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"));
      })
      .def("compute_likelihood", &GVDBInference::compute_likelihood)
      .def("get_diagnostic_image",
           [](GVDBInference& s, unsigned id, py::array out, unsigned mode) {
             s.get_diagnostic_image(id, out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"), mode);
           },
           py::arg("id"), py::arg("img"), py::arg("mode") = 0)
      .def("get_diagnostic_image_at_pose",
           [](GVDBInference& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             s.get_diagnostic_image_at_pose(pose16(pose).data(), img,
                                            out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"));
           })
      .def("get_voxel_coords",
           [](GVDBInference& s, std::vector<uint64_t> idx) {
             std::vector<float> c = s.get_voxel_coords(idx);
             py::array_t<float> a({(py::ssize_t)idx.size(), (py::ssize_t)6});
             std::copy(c.begin(), c.end(), a.mutable_data());
             return a;
           })
      .def("set_selected_x_y", &GVDBInference::set_selected_x_y)
      .def("set_selected_voxel", &GVDBInference::set_selected_voxel)
      .def("set_owned_context", [](GVDBInference&) {})
      .def("get_occupied_bricks", [](GVDBInference& s, int lev) { return bricks_array(s.get_occupied_bricks(lev)); })
      .def("get_indices_and_alphas", [](GVDBInference& s, py::array out) {
        s.get_alphas(out_buffer(out, out.ndim() == 2 ? out.shape(0) : -1, 512, "alphas"), out.shape(0), 512);
      })
      .def("get_likelihood_image_at_pose",
           [](GVDBInference& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             return s.get_likelihood_image_at_pose(pose16(pose).data(), img,
                                                   out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"));
           })
      .def("get_expected_depth_image", [](GVDBInference& s, unsigned id, py::array out) {
        s.get_expected_depth_image(id, out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"));
      })
      .def("get_accuracy_image_at_pose",
           [](GVDBInference& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             return s.get_accuracy_image_at_pose(pose16(pose).data(), img,
                                                 out_buffer(out, gvdb_params_.rows, gvdb_params_.cols, "image"));
           })
      .def("get_occupied_voxels_mask", [](GVDBInference& s, py::array out, float thr) {
        if (!py::isinstance<py::array_t<int>>(out) || out.ndim() != 2)
          throw py::type_error("mask must be a 2-D int32 array");
        s.map_->get_occupied_voxels_mask(static_cast<int*>(out.mutable_data()), out.shape(0), out.shape(1), thr);
      })
      .def_readwrite("infer_flags", &GVDBInference::infer_flags)
      .def("stats", [](GVDBInference& s) {
        mrf_stats st = s.stats();
        py::dict d;
        d["n_views"] = st.n_views;
        d["n_bricks"] = st.n_bricks;
        d["n_rays"] = st.n_rays;
        d["n_inc_pre"] = st.n_inc_pre;
        d["n_inc_post"] = st.n_inc_post;
        d["n_pairs"] = st.n_pairs;
        d["iters_done"] = st.iters_done;
        d["infer_ms"] = st.infer_ms;
        d["build_ms"] = st.build_ms;
        return d;
      });

  py::class_<GVDBMapLikelihoodEstimator, std::shared_ptr<GVDBMapLikelihoodEstimator>>(m, "GVDBMapLikelihoodEstimator")
      .def(py::init<gvdb_params_t, bool>(), py::arg("params"), py::arg("use_gl") = false)
      .def("add_camera", [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img) {
        s.add_camera(pose16(pose).data(), img);
      })
      .def("set_pose", [](GVDBMapLikelihoodEstimator& s, unsigned id, farr pose) { s.set_pose(id, pose16(pose).data()); })
      .def("activate_camera", &GVDBMapLikelihoodEstimator::activate_camera)
      .def("load_map", [](GVDBMapLikelihoodEstimator& s, farr pts, farr occ) {
        if (pts.ndim() != 2 || pts.shape(1) != 3) throw std::invalid_argument("points must be n x 3");
        if (occ.size() != pts.shape(0)) throw std::invalid_argument("occupancies must have n entries");
        return s.load_map(pts.data(), occ.data(), pts.shape(0));
      })
      .def("compute_likelihood", &GVDBMapLikelihoodEstimator::compute_likelihood)
      .def("get_likelihood_image", [](GVDBMapLikelihoodEstimator& s, unsigned id, py::array out) {
        return s.get_likelihood_image(id, out_buffer(out, s.params_.rows, s.params_.cols, "image"));
      })
      .def("get_likelihood_image_at_pose",
           [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             return s.get_likelihood_image_at_pose(pose16(pose).data(), img,
                                                   out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("get_likelihood_image_at_pose_with_depth",
           [](GVDBMapLikelihoodEstimator& s, farr pose, farr depth, py::array out) {
             check_depth(depth, s.params_);
             return s.get_likelihood_image_at_pose_with_depth(
                 pose16(pose).data(), depth.data(), out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("get_accuracy_image", [](GVDBMapLikelihoodEstimator& s, unsigned id, py::array out) {
        s.get_accuracy_image(id, out_buffer(out, s.params_.rows, s.params_.cols, "image"));
      })
      .def("get_accuracy_image_at_pose",
           [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             return s.get_accuracy_image_at_pose(pose16(pose).data(), img,
                                                 out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("get_accuracy_image_at_pose_with_depth",
           [](GVDBMapLikelihoodEstimator& s, farr pose, farr depth, py::array out) {
             check_depth(depth, s.params_);
             return s.get_accuracy_image_at_pose_with_depth(
                 pose16(pose).data(), depth.data(), out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("get_simple_accuracy_at_pose",
           [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img) {
             return s.get_simple_accuracy_at_pose(pose16(pose).data(), img);
           })
      .def("get_simple_accuracy_image_at_pose_with_depth",
           [](GVDBMapLikelihoodEstimator& s, farr pose, farr depth, py::array out) {
             check_depth(depth, s.params_);
             return s.get_simple_accuracy_image_at_pose_with_depth(
                 pose16(pose).data(), depth.data(), out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("get_occ_thresh_image_at_pose",
           [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out,
              float occ_thresh) {
             s.get_occ_thresh_image_at_pose(pose16(pose).data(), img,
                                            out_buffer(out, s.params_.rows, s.params_.cols, "image"), occ_thresh);
           })
      .def("get_diagnostic_image", [](GVDBMapLikelihoodEstimator& s, unsigned id, py::array out) {
        s.get_diagnostic_image(id, out_buffer(out, s.params_.rows, s.params_.cols, "image"));
      })
      .def("get_diagnostic_image_at_pose",
           [](GVDBMapLikelihoodEstimator& s, farr pose, std::shared_ptr<GVDBImage> img, py::array out) {
             s.get_diagnostic_image_at_pose(pose16(pose).data(), img,
                                            out_buffer(out, s.params_.rows, s.params_.cols, "image"));
           })
      .def("set_selected_x_y", &GVDBMapLikelihoodEstimator::set_selected_x_y)
      .def("set_acc_thresh", &GVDBMapLikelihoodEstimator::set_acc_thresh)
      .def("get_occupied_bricks",
           [](GVDBMapLikelihoodEstimator& s, int lev) { return bricks_array(s.get_occupied_bricks(lev)); })
      .def("get_indices_and_alphas", [](GVDBMapLikelihoodEstimator& s, py::array out) {
        s.get_alphas(out_buffer(out, out.ndim() == 2 ? out.shape(0) : -1, 512, "alphas"), out.shape(0), 512);
      });

  // src/GVDBPyModules.cpp:130-133.  compute_distance takes (rot, trans,
  // first, second) like the reference; Python cannot see the two outputs
  // through float references, so it returns rot + trans, as the reference
  // binding does.
  py::class_<KeyframeSelector>(m, "KeyframeSelector")
      .def(py::init<float, float>(), py::arg("rotation_thresh") = 0.1f, py::arg("translation_thresh") = 0.1f)
      .def("set_thresh", &KeyframeSelector::set_thresh)
      .def("is_keyframe", [](KeyframeSelector& s, farr pose) { return s.is_keyframe(pose16(pose).data()); })
      .def("compute_distance",
           [](const KeyframeSelector& s, float, float, farr a, farr b) {
             float r = 0.0f, t = 0.0f;
             return s.compute_distance(r, t, pose16(a).data(), pose16(b).data());
           })
      .def("compute_rot_trans",
           [](const KeyframeSelector& s, farr a, farr b) {
             float r = 0.0f, t = 0.0f;
             s.compute_distance(r, t, pose16(a).data(), pose16(b).data());
             return py::make_tuple(r, t);
           })
      .def("num_keyframes", &KeyframeSelector::num_keyframes);
}
