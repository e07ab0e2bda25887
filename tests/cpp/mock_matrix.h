// Stand-ins for the Eigen types the reference's C++ callers pass: a
// column-major dense matrix (Eigen::MatrixXf) and a writable row-major view
// with an outer stride (an Eigen::Ref<MRow> of a block).  Only rows(),
// cols() and m(i, j) are offered, as the shim's overloads require.
#pragma once
#include <vector>

template <class T>
struct ColMajor {
  int r, c;
  std::vector<T> v;
  ColMajor(int r_, int c_) : r(r_), c(c_), v((size_t)r_ * c_) {}
  int rows() const { return r; }
  int cols() const { return c; }
  T& operator()(int i, int j) { return v[(size_t)j * r + i]; }
  const T& operator()(int i, int j) const { return v[(size_t)j * r + i]; }
};

template <class T>
struct RowRef {
  T* p;
  int r, c, stride;
  int rows() const { return r; }
  int cols() const { return c; }
  T& operator()(int i, int j) const { return p[(size_t)i * stride + j]; }
};
