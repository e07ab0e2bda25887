// Layout conversions of the shim's matrix arguments, run on the host:
// column-major in -> row-major buffer; row-major buffer -> strided output;
// shape checks.  Prints "ok" on success.
#include <cstdio>
#include <stdexcept>

#include "mock_matrix.h"
#include "mrfmap/MatrixArgs.h"

#define REQUIRE(c)                                        \
  do {                                                    \
    if (!(c)) {                                           \
      std::printf("failed: %s (line %d)\n", #c, __LINE__); \
      return 1;                                           \
    }                                                     \
  } while (0)

int main() {
  ColMajor<float> m(3, 5);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 5; ++j) m(i, j) = 10.0f * i + j;
  std::vector<float> rm = mrf_shim::rowmajor(m);
  REQUIRE(rm.size() == 15);
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 5; ++j) REQUIRE(rm[i * 5 + j] == 10.0f * i + j);
  // a pose: the column-major storage holds the transpose's rows
  ColMajor<float> P(4, 4);
  for (int i = 0; i < 4; ++i)
    for (int j = 0; j < 4; ++j) P(i, j) = (float)(4 * i + j);
  std::vector<float> p16 = mrf_shim::pose16(P);
  for (int k = 0; k < 16; ++k) REQUIRE(p16[k] == (float)k);
  bool threw = false;
  try {
    mrf_shim::pose16(m);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  REQUIRE(threw);
  // a row-major buffer into a strided view (a block of a wider matrix)
  std::vector<float> store(3 * 8, -1.0f);
  RowRef<float> out{store.data(), 3, 5, 8};
  mrf_shim::assign(out, rm.data());
  for (int i = 0; i < 3; ++i)
    for (int j = 0; j < 8; ++j) REQUIRE(store[i * 8 + j] == (j < 5 ? 10.0f * i + j : -1.0f));
  std::vector<int> is(16, 0);
  RowRef<int> iv{is.data(), 2, 8, 8};
  const int src[16] = {1, 0, 1, 1, 0, 0, 1, 0, 0, 1, 1, 1, 0, 0, 0, 1};
  mrf_shim::assign(iv, src);
  for (int k = 0; k < 16; ++k) REQUIRE(is[k] == src[k]);
  REQUIRE(mrf_shim::image_scratch(out, 3, 5).size() == 15);
  threw = false;
  try {
    mrf_shim::image_scratch(out, 480, 640);
  } catch (const std::runtime_error&) {
    threw = true;
  }
  REQUIRE(threw);
  std::printf("ok\n");
  return 0;
}
