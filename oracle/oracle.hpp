// CPU oracle: a restatement of the prtcl reference algorithm for the hot path
// (uniform-grid neighbourhood, IISPH pressure solve, WKBB18 implicit viscosity
// PCG and the small per-step procedures around them).
//
// TEST INFRASTRUCTURE ONLY.  Only the test-suite, the smoke check and the CPU
// baseline leg of the benchmark may load this code; it is the checker, never
// the product.  The product path is the CUDA library under prtcl_gb300/.
//
// The restatement follows the reference's operation order so that FP32
// results are reproducible bit for bit by a device implementation that uses
// the same order and no fused multiply-add:
//   * vector reductions of length 3 (dot, squared norm, component sums) are
//     evaluated as  a0 + (a1 + a2)  (the halving unroller of the reference's
//     fixed-size tensor library for a 3-vector);
//   * powers are evaluated by repeated multiplication starting from 1
//     (util/constpow.hpp:9-16);
//   * every generated procedure sums its neighbours sequentially, fluid groups
//     first (ascending group index), then boundary groups, each in grid
//     traversal order.
// The build must use -ffp-contract=off (aarch64 compilers contract a*b+c by
// default; the reference is built for x86-64 without FMA).
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <map>
#include <memory>
#include <set>
#include <stdexcept>
#include <string>
#include <vector>

#include <omp.h>
#include <parallel/algorithm>

namespace oracle {

// ---------------------------------------------------------------------------
// small fixed-size tensors (math/impl/eigen.hpp semantics)
// ---------------------------------------------------------------------------

template <class T> using V3 = std::array<T, 3>;
template <class T> using M3 = std::array<T, 9>; // column-major, (r,c) -> 3c+r

template <class T> inline V3<T> vsub(V3<T> const &a, V3<T> const &b) {
  return {a[0] - b[0], a[1] - b[1], a[2] - b[2]};
}
template <class T> inline V3<T> vadd(V3<T> const &a, V3<T> const &b) {
  return {a[0] + b[0], a[1] + b[1], a[2] + b[2]};
}
template <class T> inline V3<T> vscale(T s, V3<T> const &a) {
  return {s * a[0], s * a[1], s * a[2]};
}
// dot / squaredNorm of a 3-vector: a0*b0 + (a1*b1 + a2*b2)
template <class T> inline T vdot(V3<T> const &a, V3<T> const &b) {
  return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]);
}
template <class T> inline T vnsq(V3<T> const &a) { return vdot(a, a); }
template <class T> inline T vnorm(V3<T> const &a) { return std::sqrt(vnsq(a)); }

// constpow (util/constpow.hpp:9-16): result = 1; result *= base, n times
template <class T> inline T cpow(T base, int n) {
  T r = static_cast<T>(1);
  for (; n > 0; --n) r *= base;
  return r;
}

// 3x3 inverse via the adjugate: cofactors of column 0, determinant expanded
// along column 0, then inverse(r,c) = cofactor(c,r) / det.
template <class T> inline T cof3(M3<T> const &m, int i, int j) {
  int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
  auto at = [&](int r, int c) { return m[3 * c + r]; };
  return at(i1, j1) * at(i2, j2) - at(i1, j2) * at(i2, j1);
}
template <class T> inline M3<T> minv(M3<T> const &m) {
  T c00 = cof3(m, 0, 0), c10 = cof3(m, 1, 0), c20 = cof3(m, 2, 0);
  T det = c00 * m[0] + (c10 * m[1] + c20 * m[2]);
  T invdet = T(1) / det;
  M3<T> r;
  auto set = [&](int row, int col, T v) { r[3 * col + row] = v; };
  set(0, 0, c00 * invdet);
  set(0, 1, c10 * invdet);
  set(0, 2, c20 * invdet);
  set(1, 0, cof3(m, 0, 1) * invdet);
  set(1, 1, cof3(m, 1, 1) * invdet);
  set(1, 2, cof3(m, 2, 1) * invdet);
  set(2, 0, cof3(m, 0, 2) * invdet);
  set(2, 1, cof3(m, 1, 2) * invdet);
  set(2, 2, cof3(m, 2, 2) * invdet);
  return r;
}
// matrix * vector: row_r . v  = m(r,0)v0 + (m(r,1)v1 + m(r,2)v2)
template <class T> inline V3<T> mvmul(M3<T> const &m, V3<T> const &v) {
  V3<T> r;
  for (int i = 0; i < 3; ++i)
    r[i] = m[i] * v[0] + (m[3 + i] * v[1] + m[6 + i] * v[2]);
  return r;
}

// unit_step_l (math/impl/eigen.hpp:307-314): 1 if eps < x else 0
// Moore-Penrose pseudo-inverse of a 3x3 matrix (column-major m[3 c + r]):
// one-sided Jacobi SVD (Hestenes) with a fixed 8 sweeps over the column pairs
// (0,1), (0,2), (1,2); A V = W with orthogonal columns w_i = sigma_i u_i, so
// A+ = sum_i v_i w_i^T / sigma_i^2 over the sigma_i > 3 eps sigma_max (the
// rank threshold of a complete orthogonal decomposition of a 3x3 matrix).
// Stands in for the reference's invert_pm (math/impl/eigen.hpp:266-276,
// Eigen's completeOrthogonalDecomposition().pseudoInverse()); agrees with it
// to rounding where the rank is clear.
template <class T> inline T dot3r(T const *a, T const *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
template <class T> inline M3<T> pinv3(M3<T> const &A) {
  T w[3][3], v[3][3];
  for (int c = 0; c < 3; ++c)
    for (int r = 0; r < 3; ++r) {
      w[c][r] = A[3 * c + r];
      v[c][r] = (r == c) ? T(1) : T(0);
    }
  static constexpr int pairs[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 8; ++sweep)
    for (auto const &pq : pairs) {
      int p = pq[0], q = pq[1];
      T alpha = dot3r(w[p], w[p]), beta = dot3r(w[q], w[q]), gamma = dot3r(w[p], w[q]);
      if (gamma == T(0)) continue;
      T zeta = (beta - alpha) / (T(2) * gamma);
      T t = std::copysign(T(1), zeta) / (std::fabs(zeta) + std::sqrt(T(1) + zeta * zeta));
      T c = T(1) / std::sqrt(T(1) + t * t);
      T s = c * t;
      for (int r = 0; r < 3; ++r) {
        T wp = w[p][r], wq = w[q][r];
        w[p][r] = c * wp - s * wq;
        w[q][r] = s * wp + c * wq;
        T vp = v[p][r], vq = v[q][r];
        v[p][r] = c * vp - s * vq;
        v[q][r] = s * vp + c * vq;
      }
    }
  T s2[3], smax = T(0);
  for (int i = 0; i < 3; ++i) {
    s2[i] = dot3r(w[i], w[i]);
    T si = std::sqrt(s2[i]);
    if (si > smax) smax = si;
  }
  T thr = T(3) * std::numeric_limits<T>::epsilon() * smax;
  M3<T> R;
  R.fill(T(0));
  for (int i = 0; i < 3; ++i) {
    if (!(std::sqrt(s2[i]) > thr)) continue;
    for (int c = 0; c < 3; ++c)
      for (int r = 0; r < 3; ++r) R[3 * c + r] = R[3 * c + r] + (v[i][r] * w[i][c]) / s2[i];
  }
  return R;
}

template <class T> inline T ustep(T eps, T x) { return (eps < x) ? T(1) : T(0); }
// reciprocal_or_zero (math/impl/eigen.hpp:293-300)
template <class T> inline T rcp0(T x, T eps) {
  return (std::abs(x) > eps) ? T(1) / x : T(0);
}

// ---------------------------------------------------------------------------
// cubic spline kernel, support 2h
// (math/kernel/cubic_spline_kernel.hpp:43-102, kernel_facade.hpp:95-120)
// ---------------------------------------------------------------------------

template <class T> struct Kernel {
  T h, h3, h4, sigma, eps;
  explicit Kernel(T h_) : h(h_) {
    h3 = cpow(h, 3);
    h4 = cpow(h, 4);
    sigma = static_cast<T>(0.25L * 0.318309886183790671537767526745028724L);
    eps = std::sqrt(std::numeric_limits<T>::epsilon());
  }
  T evalq(T q) const {
    T result = 0;
    if (q < 1) result -= 4 * cpow(T(1) - q, 3);
    if (q < 2) result += cpow(T(2) - q, 3);
    return sigma * result;
  }
  T evaldq(T q) const {
    T result = 0;
    if (q < 1) result += 12 * cpow(T(1) - q, 2);
    if (q < 2) result -= 3 * cpow(T(2) - q, 2);
    return sigma * result;
  }
  T evalr(T r) const { return evalq(std::abs(r) / h) / h3; }
  T evaldr(T r) const { return -std::copysign(evaldq(std::abs(r) / h) / h4, r); }
  T W(V3<T> const &v) const { return evalr(vnorm(v)); }
  V3<T> gradW(V3<T> const &v) const {
    T r = vnorm(v);
    if (r < eps) return {T(0), T(0), T(0)};
    return vscale(evaldr(r) / r, v);
  }
};

// ---------------------------------------------------------------------------
// Morton (Z-curve) order without building keys (util/morton_order.hpp:40-82)
// ---------------------------------------------------------------------------

using GI = std::array<int32_t, 3>;

inline uint32_t unsign(int32_t i) {
  // (uint32)i + INT32_MAX, modulo 2^32 (the reference's bias, not i ^ 2^31)
  return static_cast<uint32_t>(i) + 0x7FFFFFFFu;
}
inline bool less_msb(uint32_t a, uint32_t b) { return a < b && a < (a ^ b); }
inline int morton_compare(GI const &l, GI const &r) {
  int msd = 0;
  for (int d = 1; d < 3; ++d)
    if (less_msb(unsign(l[msd]) ^ unsign(r[msd]), unsign(l[d]) ^ unsign(r[d])))
      msd = d;
  uint32_t a = unsign(l[msd]), b = unsign(r[msd]);
  return a < b ? -1 : (a > b ? 1 : 0);
}
inline bool morton_less(GI const &l, GI const &r) { return morton_compare(l, r) < 0; }

// the 13 half-stencil offsets (util/grouped_uniform_grid.hpp:52-68); slot k
// of a cell holds the cell at +offset[k], slot 25-k the cell at -offset[k]
static constexpr int32_t kOffsets[13][3] = {
    {1, 0, 0},  {0, 1, 0},  {0, 0, 1},   {1, 1, 0},   {1, 0, 1},
    {0, 1, 1},  {1, 1, 1},  {0, -1, 1},  {1, 0, -1},  {1, 1, -1},
    {1, -1, -1}, {1, -1, 0}, {1, -1, 1}};

// ---------------------------------------------------------------------------
// data model mirror (data/model.cpp:13-34, data/varying_field.hpp:26-58)
// ---------------------------------------------------------------------------

template <class T> struct Field {
  int ncomp = 1; // 1 (real), 3 (real[]), 9 (real[][] column-major)
  std::vector<T> data;
};

template <class T> struct Group {
  std::string name, type;
  std::set<std::string> tags;
  size_t count = 0;
  std::map<std::string, Field<T>> varying;
  std::map<std::string, std::vector<double>> uniform;

  bool has_tag(std::string const &t) const { return tags.count(t) > 0; }
  Field<T> &vf(std::string const &n, int ncomp) {
    auto it = varying.find(n);
    if (it == varying.end()) {
      Field<T> f;
      f.ncomp = ncomp;
      f.data.assign(count * ncomp, T(0));
      it = varying.emplace(n, std::move(f)).first;
    }
    if (it->second.ncomp != ncomp) throw std::runtime_error("field of different type already exists: " + n);
    return it->second;
  }
  std::vector<double> &uf(std::string const &n, int ncomp) {
    auto it = uniform.find(n);
    if (it == uniform.end()) it = uniform.emplace(n, std::vector<double>(ncomp, 0.0)).first;
    return it->second;
  }
  V3<T> *v3(std::string const &n) { return reinterpret_cast<V3<T> *>(vf(n, 3).data.data()); }
  T *s1(std::string const &n) { return vf(n, 1).data.data(); }
  M3<T> *m3(std::string const &n) { return reinterpret_cast<M3<T> *>(vf(n, 9).data.data()); }
};

// ---------------------------------------------------------------------------
// grouped uniform grid (util/grouped_uniform_grid.hpp) + Neighborhood
// (util/neighborhood.cpp:61-166)
// ---------------------------------------------------------------------------

inline uint32_t pack_handle(size_t g, size_t i) { return (uint32_t(g) << 28) | uint32_t(i); }
inline size_t handle_group(uint32_t h) { return h >> 28; }
inline size_t handle_index(uint32_t h) { return h & 0x0FFFFFFFu; }

template <class T> struct Grid {
  double radius = 1.0;
  // per group: position span (nullptr if the group has no position field)
  std::vector<V3<T> const *> pos;
  std::vector<size_t> count;
  std::vector<bool> can_be_neighbor;

  std::vector<uint32_t> sorted_to_raw;
  std::vector<std::vector<int32_t>> raw_to_sorted;
  std::vector<int32_t> sorted_to_cell;
  std::vector<std::array<int32_t, 2>> cell_range;
  std::vector<GI> cell_gi;
  std::vector<std::array<int32_t, 26>> cell_adj;

  GI x_to_gi(V3<T> const &x) const {
    GI r;
    for (int a = 0; a < 3; ++a)
      r[a] = static_cast<int32_t>(std::floor(static_cast<double>(x[a]) / radius));
    return r;
  }
  GI handle_gi(uint32_t h) const { return x_to_gi(pos[handle_group(h)][handle_index(h)]); }

  void update();
  int32_t find_cell(GI const &gi) const {
    auto it = std::lower_bound(cell_gi.begin(), cell_gi.end(), gi, morton_less);
    if (it == cell_gi.end() || *it != gi) return -1;
    return static_cast<int32_t>(it - cell_gi.begin());
  }
  template <class Fn> void visit_cell(int32_t c, Fn &&fn) const {
    if (c < 0) return;
    for (int32_t s = cell_range[c][0]; s < cell_range[c][1]; ++s) {
      uint32_t h = sorted_to_raw[s];
      fn(handle_group(h), handle_index(h));
    }
  }
  // grouped_uniform_grid::neighbors (util/grouped_uniform_grid.hpp:407-422,
  // 471-531): every (group, raw index) of the stencil with d^2 < r^2
  template <class Fn> void neighbors(size_t g, size_t i, Fn &&fn) const {
    if (!pos[g]) return; // CopyNeighbors skips groups without position
    double const r2 = radius * radius;
    V3<T> const xi = pos[g][i];
    auto filt = [&](size_t ng, size_t ni) {
      T d = vnsq(vsub(xi, pos[ng][ni]));
      if (static_cast<double>(d) < r2) fn(ng, ni);
    };
    if (can_be_neighbor[g]) {
      int32_t c = sorted_to_cell[raw_to_sorted[g][i]];
      visit_cell(c, filt);
      for (int k = 0; k < 26; ++k) visit_cell(cell_adj[c][k], filt);
    } else {
      GI gi = x_to_gi(xi);
      int32_t c = find_cell(gi);
      if (c >= 0) {
        visit_cell(c, filt);
        for (int k = 0; k < 26; ++k) visit_cell(cell_adj[c][k], filt);
      } else {
        for (int k = 0; k < 13; ++k) {
          GI y = gi;
          for (int a = 0; a < 3; ++a) y[a] += kOffsets[k][a];
          visit_cell(find_cell(y), filt);
          for (int a = 0; a < 3; ++a) y[a] -= 2 * kOffsets[k][a];
          visit_cell(find_cell(y), filt);
        }
      }
    }
  }
};

template <class T> void Grid<T>::update() {
  size_t G = pos.size();
  raw_to_sorted.assign(G, {});
  // group-major identity order over the groups that can be neighbours
  sorted_to_raw.clear();
  for (size_t g = 0; g < G; ++g) {
    if (!can_be_neighbor[g] || !pos[g]) continue;
    if (count[g] >= (size_t(1) << 28)) throw std::runtime_error("group too large for the grid (>= 2^28 items)");
    raw_to_sorted[g].assign(count[g], -1);
    for (size_t i = 0; i < count[g]; ++i) sorted_to_raw.push_back(pack_handle(g, i));
  }
  if (G > 16) throw std::runtime_error("too many groups for the grid (> 16)");
  // Morton order of the cell; ties (same cell) broken by (group, raw index).
  // The reference's parallel sort is unstable, so its within-cell order is
  // unspecified; the oracle fixes it to this deterministic tie-break.
  auto cmp = [this](uint32_t a, uint32_t b) {
    int c = morton_compare(handle_gi(a), handle_gi(b));
    if (c != 0) return c < 0;
    return a < b;
  };
  // a parallel comparison sort, as the reference's block_indirect_sort
  __gnu_parallel::sort(sorted_to_raw.begin(), sorted_to_raw.end(), cmp);
  size_t N = sorted_to_raw.size();
#pragma omp parallel for
  for (size_t s = 0; s < N; ++s) {
    uint32_t h = sorted_to_raw[s];
    raw_to_sorted[handle_group(h)][handle_index(h)] = static_cast<int32_t>(s);
  }
  // cell boundaries, then a serial scan (util/grouped_uniform_grid.hpp:220-306)
  sorted_to_cell.assign(N, 0);
  cell_range.clear();
  cell_gi.clear();
  cell_adj.clear();
  if (N == 0) return;
  std::vector<GI> sgi(N);
#pragma omp parallel for
  for (size_t s = 0; s < N; ++s) sgi[s] = handle_gi(sorted_to_raw[s]);
  cell_range.push_back({0, 0});
  cell_gi.push_back(sgi[0]);
  for (size_t s = 1; s < N; ++s) {
    int32_t c = sorted_to_cell[s - 1];
    if (sgi[s] != sgi[s - 1]) {
      cell_range[c][1] = static_cast<int32_t>(s);
      c += 1;
      cell_range.push_back({static_cast<int32_t>(s), 0});
      cell_gi.push_back(sgi[s]);
    }
    sorted_to_cell[s] = c;
  }
  cell_range.back()[1] = static_cast<int32_t>(N);
  size_t C = cell_gi.size();
  std::array<int32_t, 26> none;
  none.fill(-1);
  cell_adj.assign(C, none);
  // adjacency (util/grouped_uniform_grid.hpp:312-337): slot k and mirror 25-k
#pragma omp parallel for
  for (size_t c = 0; c < C; ++c) {
    for (int k = 0; k < 13; ++k) {
      GI y = cell_gi[c];
      for (int a = 0; a < 3; ++a) y[a] += kOffsets[k][a];
      int32_t j = find_cell(y);
      if (j >= 0) {
        cell_adj[c][k] = j;
        cell_adj[j][25 - k] = static_cast<int32_t>(c);
      }
    }
  }
}

} // namespace oracle
