// Test infrastructure, not part of the library: a thin C wrapper around the
// reference's own Morton comparison (prtcl/util/morton_order.hpp:19-95),
// compiled from the reference source tree by ref_build.py into
// oracle/_ref/libref_morton.so.  It is the one piece of the reference's hot
// path that builds from its own sources (the grid needs Boost.Sort and the
// kernel needs Eigen and a generated config header); the fixtures in
// tests/golden/ that pin the oracle's Morton order are made with it.
#include <algorithm>
#include <array>
#include <cstdint>
#include <limits>
#include <numeric>
#include <vector>

#include "prtcl/util/morton_order.hpp"

using Triple = std::array<int32_t, 3>;

static Triple at(int32_t const *p, int64_t i) { return {p[3 * i], p[3 * i + 1], p[3 * i + 2]}; }

extern "C" {

// three-way compare of n pairs, through morton_order_fn::compare
void ref_morton_compare_many(int32_t const *a, int32_t const *b, int64_t n, int8_t *out) {
  for (int64_t i = 0; i < n; ++i) out[i] = int8_t(prtcl::morton_order.compare(at(a, i), at(b, i)));
}

// order of n triples under morton_order_fn::operator() (a strict weak order
// on distinct triples); equal triples keep their input order
void ref_morton_sort(int32_t const *gi, int64_t n, int64_t *order) {
  std::vector<int64_t> o(static_cast<size_t>(n));
  std::iota(o.begin(), o.end(), int64_t(0));
  std::stable_sort(o.begin(), o.end(), [&](int64_t x, int64_t y) { return prtcl::morton_order(at(gi, x), at(gi, y)); });
  std::copy(o.begin(), o.end(), order);
}
}
