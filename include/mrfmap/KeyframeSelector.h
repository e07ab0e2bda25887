// KeyframeSelector.h -- keyframe selection by SE(3) distance
// (reference include/mrfmap/KeyframeSelector.h:5-19,
// src/KeyframeSelector.cpp:74-99).  Poses are row-major 4x4
// camera-to-world matrices (16 floats).  Host code only.
#pragma once
#include <array>
#include <vector>

class KeyframeSelector {
 public:
  explicit KeyframeSelector(float rotation_thresh = 0.1f, float translation_thresh = 0.1f)
      : rotation_thresh_(rotation_thresh), translation_thresh_(translation_thresh) {}
  void set_thresh(float rot_thresh, float trans_thresh) {
    rotation_thresh_ = rot_thresh;
    translation_thresh_ = trans_thresh;
  }
  // True (and the pose is kept) unless some kept keyframe lies within both
  // thresholds of it.
  bool is_keyframe(const float* pose);
  // Tangent-space distance of the relative motion first^-1 * second: rot =
  // |rotation vector| (rad), trans = |translation part of the SE(3)
  // logarithm|; returns rot + trans.
  float compute_distance(float& rot, float& trans, const float* first, const float* second) const;
  size_t num_keyframes() const { return kf_poses_.size(); }

 private:
  float rotation_thresh_, translation_thresh_;
  std::vector<std::array<float, 16>> kf_poses_;
};
