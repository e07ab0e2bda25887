// MatrixArgs.h -- matrix arguments of the reference's C++ API without a
// dependency on Eigen.
//
// The reference passes poses and depth images as Eigen::MatrixXf (column
// major) and returns images through Eigen::Ref<MRow> (row major)
// (include/mrfmap/GVDBInference.h:87-102,
// include/mrfmap/GVDBMapLikelihoodEstimator.h:97-117).  The shim classes take
// row-major float buffers; the template overloads in the class headers
// accept any matrix type that offers rows(), cols() and element access
// m(i, j) -- Eigen matrices, maps and Refs among them -- so a reference
// caller compiles unchanged.  Elements are copied through m(i, j), which
// makes the storage order and strides of the caller's type irrelevant.
#pragma once
#include <cstdint>
#include <stdexcept>
#include <type_traits>
#include <utility>
#include <vector>

namespace mrf_shim {

// enabled for types with rows(), cols() and a readable m(i, j)
template <class M>
using if_matrix = decltype((void)std::declval<const M&>().rows(), (void)std::declval<const M&>().cols(),
                           (void)static_cast<float>(std::declval<const M&>()(0, 0)));

// the same, for an output with a writable m(i, j)
template <class M>
using if_out_matrix = decltype((void)std::declval<M&>().rows(), (void)std::declval<M&>().cols(),
                               (void)(std::declval<M&>()(0, 0) = 0.0f));

// rows x cols elements of m in row-major order
template <class M, class = if_matrix<M>>
std::vector<float> rowmajor(const M& m) {
  const int64_t r = (int64_t)m.rows(), c = (int64_t)m.cols();
  std::vector<float> out((size_t)(r * c));
  for (int64_t i = 0; i < r; ++i)
    for (int64_t j = 0; j < c; ++j) out[(size_t)(i * c + j)] = static_cast<float>(m((int)i, (int)j));
  return out;
}

// a 4x4 pose in row-major order (throws on another shape)
template <class M, class = if_matrix<M>>
std::vector<float> pose16(const M& m) {
  if (m.rows() != 4 || m.cols() != 4) throw std::runtime_error("pose must be a 4x4 matrix");
  return rowmajor(m);
}

// a row-major buffer of out.rows() x out.cols() written into out
template <class M, class T>
void assign(M& out, const T* src) {
  const int64_t r = (int64_t)out.rows(), c = (int64_t)out.cols();
  for (int64_t i = 0; i < r; ++i)
    for (int64_t j = 0; j < c; ++j) out((int)i, (int)j) = src[(size_t)(i * c + j)];
}

// row-major scratch for an output image of the camera's rows x cols (the
// reference writes the camera's image size; throws on another shape)
template <class M>
std::vector<float> image_scratch(const M& out, int rows, int cols) {
  if ((int64_t)out.rows() != rows || (int64_t)out.cols() != cols)
    throw std::runtime_error("output image must have the camera's rows x cols");
  return std::vector<float>((size_t)rows * (size_t)cols);
}

template <class M>
using plain = typename std::remove_cv<typename std::remove_reference<M>::type>::type;

}  // namespace mrf_shim
