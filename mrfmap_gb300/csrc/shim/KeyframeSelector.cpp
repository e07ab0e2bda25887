// KeyframeSelector.cpp -- SE(3) logarithm of the relative motion between two
// poses (the same quantity the reference computes, src/KeyframeSelector.cpp:
// 4-72, restated from the Lie-group formulas: for R = exp([w]x) with angle
// t = |w|, the translation part of log(T) is V^-1 p with
// V^-1 = I - [w]x / 2 + (1 - t / (2 tan(t/2))) [w]x^2 / t^2).  Double
// precision throughout.
#include "mrfmap/KeyframeSelector.h"

#include <cmath>

namespace {

struct Mat3 {
  double a[3][3];
};

// rotation vector of a rotation matrix: angle t = atan2(|v|/2, (tr-1)/2)
// with v = vee(R - R^T) (well conditioned at every angle), direction v/|v|;
// near t = pi, where v vanishes, the axis comes from R + I = 2 u u^T
void log_so3(const Mat3& R, double w[3]) {
  const double tr = R.a[0][0] + R.a[1][1] + R.a[2][2];
  const double v[3] = {R.a[2][1] - R.a[1][2], R.a[0][2] - R.a[2][0], R.a[1][0] - R.a[0][1]};
  const double sn = 0.5 * std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
  const double t = std::atan2(sn, 0.5 * (tr - 1.0));
  if (t < 1e-6) {  // w = v / 2 to first order
    for (int j = 0; j < 3; ++j) w[j] = 0.5 * v[j];
    return;
  }
  if (sn > 1e-4) {
    for (int j = 0; j < 3; ++j) w[j] = t * v[j] / (2.0 * sn);
    return;
  }
  int i = 0;
  for (int j = 1; j < 3; ++j)
    if (R.a[j][j] > R.a[i][i]) i = j;
  double u[3];
  const double d = std::sqrt(std::fmax(0.0, 0.5 * (R.a[i][i] + 1.0)));
  for (int j = 0; j < 3; ++j) u[j] = (j == i) ? d : 0.5 * (R.a[i][j] + R.a[j][i]) / (2.0 * d);
  const double n = std::sqrt(u[0] * u[0] + u[1] * u[1] + u[2] * u[2]);
  // orient the axis by the (small) antisymmetric part where it is defined
  const double sgn = (u[0] * v[0] + u[1] * v[1] + u[2] * v[2] < 0.0) ? -1.0 : 1.0;
  for (int j = 0; j < 3; ++j) w[j] = sgn * t * u[j] / n;
}

}  // namespace

float KeyframeSelector::compute_distance(float& rot, float& trans, const float* first,
                                         const float* second) const {
  // delta = first^-1 * second for rigid transforms: R = R1^T R2, p = R1^T (p2 - p1)
  Mat3 R{};
  double p[3] = {0.0, 0.0, 0.0};
  for (int r = 0; r < 3; ++r) {
    for (int c = 0; c < 3; ++c) {
      double acc = 0.0;
      for (int k = 0; k < 3; ++k) acc += (double)first[k * 4 + r] * (double)second[k * 4 + c];
      R.a[r][c] = acc;
    }
    for (int k = 0; k < 3; ++k) p[r] += (double)first[k * 4 + r] * ((double)second[k * 4 + 3] - first[k * 4 + 3]);
  }
  double w[3];
  log_so3(R, w);
  const double t2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
  const double t = std::sqrt(t2);
  // u = V^-1 p
  const double wp[3] = {w[1] * p[2] - w[2] * p[1], w[2] * p[0] - w[0] * p[2], w[0] * p[1] - w[1] * p[0]};
  const double wwp[3] = {w[1] * wp[2] - w[2] * wp[1], w[2] * wp[0] - w[0] * wp[2], w[0] * wp[1] - w[1] * wp[0]};
  double b;  // (1 - t / (2 tan(t/2))) / t^2, -> 1/12 as t -> 0
  if (t < 1e-4)
    b = 1.0 / 12.0 + t2 / 720.0;
  else
    b = (1.0 - t / (2.0 * std::tan(0.5 * t))) / t2;
  double u2 = 0.0;
  for (int j = 0; j < 3; ++j) {
    const double uj = p[j] - 0.5 * wp[j] + b * wwp[j];
    u2 += uj * uj;
  }
  rot = (float)t;
  trans = (float)std::sqrt(u2);
  return rot + trans;
}

bool KeyframeSelector::is_keyframe(const float* pose) {
  for (auto it = kf_poses_.rbegin(); it != kf_poses_.rend(); ++it) {
    float rot = 0.0f, trans = 0.0f;
    compute_distance(rot, trans, pose, it->data());
    if (trans < translation_thresh_ && rot < rotation_thresh_) return false;
  }
  std::array<float, 16> p;
  for (int k = 0; k < 16; ++k) p[k] = pose[k];
  kf_poses_.push_back(p);
  return true;
}
