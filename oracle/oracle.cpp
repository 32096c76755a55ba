// CPU oracle (TEST INFRASTRUCTURE ONLY): scene, generated-procedure
// restatements, the step loop and a C ABI for the test-suite.
//
// Procedures restated here, each following the reference's generated code:
//   density.compute_density            schemes/density.hpp:160-220
//   sesph.compute_density_and_pressure schemes/sesph.hpp:171-237
//   sesph.accumulate_acceleration      schemes/sesph.hpp:240-302
//   aiast12.compute_volume             schemes/aiast12.hpp:125-175
//   gravity.initialize_acceleration    schemes/gravity.hpp:133-158
//   symplectic_euler.integrate_velocity_with_hard_fade
//                                      schemes/symplectic_euler.hpp:172-201
//   symplectic_euler.integrate_position schemes/symplectic_euler.hpp:236-270
//   iisph.setup                        schemes/iisph.hpp:188-355
//   iisph.iteration_pressure_acceleration schemes/iisph.hpp:358-423
//   iisph.iteration_pressure           schemes/iisph.hpp:426-516
//   wkbb18.compute_diagonal            schemes/wkbb18.hpp:194-270
//   wkbb18.accumulate_acceleration     schemes/wkbb18.hpp:273-425 with the
//                                      solver solver/cg_openmp.hpp:35-236
// Step loop: share/scripts/prtcl-lua.example.lua:363-461.
//
// Two reduction modes:
//   reference mode: the density-error sum and the CG dot products are
//     accumulated in T by an OpenMP reduction, as the generated code does
//     (order depends on the thread count);
//   FP64 mode: per-item contributions are computed in T exactly as above and
//     accumulated sequentially in double (deterministic).  The device path
//     implements this mode.
#include "oracle.hpp"

#include <cstdio>
#include <functional>

namespace oracle {

struct SceneBase {
  virtual ~SceneBase() = default;
  virtual int real_bytes() const = 0;
  virtual void add_group(std::string const &name, std::string const &type) = 0;
  virtual void add_tag(std::string const &g, std::string const &tag) = 0;
  virtual void resize(std::string const &g, size_t n) = 0;
  virtual size_t group_count() const = 0;
  virtual int group_index(std::string const &g) const = 0;
  virtual size_t item_count(std::string const &g) const = 0;
  virtual void set_varying(std::string const &g, std::string const &f, int ncomp, void const *data, size_t n) = 0;
  virtual void get_varying(std::string const &g, std::string const &f, int ncomp, void *data, size_t n) = 0;
  virtual void set_uniform(std::string const &g, std::string const &f, double const *v, int n) = 0;
  virtual void get_uniform(std::string const &g, std::string const &f, double *v, int n) = 0;
  virtual void set_global(std::string const &f, double const *v, int n) = 0;
  virtual void get_global(std::string const &f, double *v, int n) = 0;
  virtual void set_radius(double r) = 0;
  virtual void nhood_load() = 0;
  virtual void nhood_update() = 0;
  virtual void nhood_permute() = 0;
  virtual void run(std::string const &scheme, std::string const &proc) = 0;
  virtual size_t grid_sorted_count() const = 0;
  virtual size_t grid_cell_count() const = 0;
  virtual void grid_dump(uint32_t *sorted, int32_t *cell_gi, int32_t *cell_range, int32_t *cell_adj) const = 0;
  virtual size_t neighbors(int g, size_t i, int64_t *counts, int64_t *out, size_t cap) const = 0;
  virtual void neighbor_lists(int qg, int ng, int64_t *offsets, uint32_t *idx, size_t cap) const = 0;
  bool fp64 = true;
};

template <class T> struct Scene : SceneBase {
  using R = T;
  std::map<std::string, std::vector<double>> global;
  std::vector<Group<T>> groups; // ordered by name: index = alphabetical rank
  Grid<T> grid;
  double radius = 1.0;
  bool loaded = false;

  int real_bytes() const override { return sizeof(T); }

  Group<T> &G(std::string const &n) {
    for (auto &g : groups)
      if (g.name == n) return g;
    throw std::runtime_error("group not found: " + n);
  }
  Group<T> const &G(std::string const &n) const {
    for (auto &g : groups)
      if (g.name == n) return g;
    throw std::runtime_error("group not found: " + n);
  }
  void add_group(std::string const &name, std::string const &type) override {
    for (auto &g : groups)
      if (g.name == name) {
        if (g.type != type) throw std::runtime_error("group of different type already exists");
        return;
      }
    Group<T> g;
    g.name = name;
    g.type = type;
    groups.push_back(std::move(g));
    std::sort(groups.begin(), groups.end(), [](auto const &a, auto const &b) { return a.name < b.name; });
  }
  void add_tag(std::string const &g, std::string const &tag) override { G(g).tags.insert(tag); }
  void resize(std::string const &gn, size_t n) override {
    auto &g = G(gn);
    g.count = n;
    for (auto &kv : g.varying) kv.second.data.resize(n * kv.second.ncomp, T(0));
  }
  size_t group_count() const override { return groups.size(); }
  int group_index(std::string const &gn) const override {
    for (size_t i = 0; i < groups.size(); ++i)
      if (groups[i].name == gn) return int(i);
    return -1;
  }
  size_t item_count(std::string const &g) const override { return G(g).count; }
  void set_varying(std::string const &gn, std::string const &f, int ncomp, void const *data, size_t n) override {
    auto &g = G(gn);
    if (n != g.count) throw std::runtime_error("item count mismatch for " + f);
    auto &fl = g.vf(f, ncomp);
    std::memcpy(fl.data.data(), data, n * ncomp * sizeof(T));
  }
  void get_varying(std::string const &gn, std::string const &f, int ncomp, void *data, size_t n) override {
    auto &g = G(gn);
    if (n != g.count) throw std::runtime_error("item count mismatch for " + f);
    auto &fl = g.vf(f, ncomp);
    std::memcpy(data, fl.data.data(), n * ncomp * sizeof(T));
  }
  void set_uniform(std::string const &gn, std::string const &f, double const *v, int n) override {
    G(gn).uniform[f] = std::vector<double>(v, v + n);
  }
  void get_uniform(std::string const &gn, std::string const &f, double *v, int n) override {
    auto &u = G(gn).uf(f, n);
    for (int k = 0; k < n; ++k) v[k] = u[k];
  }
  void set_global(std::string const &f, double const *v, int n) override { global[f] = std::vector<double>(v, v + n); }
  void get_global(std::string const &f, double *v, int n) override {
    auto &u = gl(f, n);
    for (int k = 0; k < n; ++k) v[k] = u[k];
  }
  std::vector<double> &gl(std::string const &f, int n) {
    auto it = global.find(f);
    if (it == global.end()) it = global.emplace(f, std::vector<double>(n, 0.0)).first;
    return it->second;
  }
  T gr(std::string const &f) { return static_cast<T>(gl(f, 1)[0]); }
  V3<T> gv(std::string const &f) {
    auto &v = gl(f, 3);
    return {static_cast<T>(v[0]), static_cast<T>(v[1]), static_cast<T>(v[2])};
  }
  T ur(Group<T> &g, std::string const &f) { return static_cast<T>(g.uf(f, 1)[0]); }

  // ---- neighbourhood -------------------------------------------------------
  void set_radius(double r) override { radius = r; }
  void nhood_load() override {
    size_t Gn = groups.size();
    grid.pos.assign(Gn, nullptr);
    grid.count.assign(Gn, 0);
    grid.can_be_neighbor.assign(Gn, false);
    for (size_t g = 0; g < Gn; ++g) {
      auto &gr_ = groups[g];
      auto it = gr_.varying.find("position");
      if (it != gr_.varying.end() && it->second.ncomp == 3) {
        grid.pos[g] = reinterpret_cast<V3<T> const *>(it->second.data.data());
        grid.count[g] = gr_.count;
      }
      grid.can_be_neighbor[g] = !gr_.has_tag("cannot_be_neighbor");
    }
    loaded = true;
  }
  void nhood_update() override {
    if (!loaded) nhood_load();
    // refresh spans (fields may have been reallocated)
    nhood_load();
    grid.radius = radius;
    grid.update();
  }
  // Neighborhood::Permute (util/neighborhood.cpp:106-154): gather every
  // varying field of each neighbour-capable group into sorted order.
  void nhood_permute() override {
    size_t Gn = groups.size();
    std::vector<std::vector<size_t>> perm(Gn);
    for (size_t g = 0; g < Gn; ++g) {
      perm[g].resize(groups[g].count);
      for (size_t i = 0; i < perm[g].size(); ++i) perm[g][i] = i;
    }
    std::vector<size_t> fill(Gn, 0);
    for (uint32_t h : grid.sorted_to_raw) {
      size_t g = handle_group(h);
      perm[g][fill[g]++] = handle_index(h);
    }
    for (size_t g = 0; g < Gn; ++g) {
      if (groups[g].has_tag("cannot_be_neighbor")) continue;
      for (auto &kv : groups[g].varying) {
        auto &f = kv.second;
        std::vector<T> nd(f.data.size());
        int nc = f.ncomp;
        for (size_t i = 0; i < groups[g].count; ++i)
          for (int c = 0; c < nc; ++c) nd[i * nc + c] = f.data[perm[g][i] * nc + c];
        f.data.swap(nd);
      }
    }
    nhood_update();
  }
  size_t grid_sorted_count() const override { return grid.sorted_to_raw.size(); }
  size_t grid_cell_count() const override { return grid.cell_gi.size(); }
  void grid_dump(uint32_t *sorted, int32_t *cell_gi, int32_t *cell_range, int32_t *cell_adj) const override {
    size_t N = grid.sorted_to_raw.size(), C = grid.cell_gi.size();
    if (sorted) std::memcpy(sorted, grid.sorted_to_raw.data(), N * 4);
    for (size_t c = 0; c < C; ++c) {
      if (cell_gi)
        for (int a = 0; a < 3; ++a) cell_gi[3 * c + a] = grid.cell_gi[c][a];
      if (cell_range)
        for (int a = 0; a < 2; ++a) cell_range[2 * c + a] = grid.cell_range[c][a];
      if (cell_adj)
        for (int a = 0; a < 26; ++a) cell_adj[26 * c + a] = grid.cell_adj[c][a];
    }
  }
  size_t neighbors(int g, size_t i, int64_t *counts, int64_t *out, size_t cap) const override {
    size_t Gn = groups.size();
    std::vector<std::vector<size_t>> nb(Gn);
    grid.neighbors(size_t(g), i, [&](size_t ng, size_t ni) { nb[ng].push_back(ni); });
    size_t k = 0;
    for (size_t q = 0; q < Gn; ++q) {
      counts[q] = int64_t(nb[q].size());
      for (size_t j : nb[q]) {
        if (k < cap) out[k] = int64_t(j);
        ++k;
      }
    }
    return k;
  }
  // CSR lists of (query group qg) -> (neighbour group ng) neighbours, in
  // traversal order; offsets has count+1 entries
  void neighbor_lists(int qg, int ng, int64_t *offsets, uint32_t *idx, size_t cap) const override {
    size_t n = groups[qg].count;
    std::vector<std::vector<uint32_t>> all(n);
#pragma omp parallel for schedule(dynamic, 256)
    for (size_t i = 0; i < n; ++i)
      grid.neighbors(size_t(qg), i, [&](size_t g2, size_t j) {
        if (int(g2) == ng) all[i].push_back(uint32_t(j));
      });
    offsets[0] = 0;
    for (size_t i = 0; i < n; ++i) offsets[i + 1] = offsets[i] + int64_t(all[i].size());
    if (size_t(offsets[n]) > cap) throw std::runtime_error("neighbor_lists: capacity too small");
    for (size_t i = 0; i < n; ++i) std::copy(all[i].begin(), all[i].end(), idx + offsets[i]);
  }

  // ---- procedure helpers ---------------------------------------------------
  std::vector<Group<T> *> of_type(char const *type) {
    std::vector<Group<T> *> r;
    for (auto &g : groups)
      if (g.type == type) r.push_back(&g);
    return r;
  }
  std::vector<Group<T> *> with_tag(char const *tag) {
    std::vector<Group<T> *> r;
    for (auto &g : groups)
      if (g.has_tag(tag)) r.push_back(&g);
    return r;
  }
  size_t gidx(Group<T> *g) const { return size_t(g - groups.data()); }

  // foreach particle of `gs`, with per-thread neighbour storage re-filled for
  // every particle (the generated code's CopyNeighbors per particle)
  template <class Fn> void foreach_with_neighbors(std::vector<Group<T> *> const &gs, Fn &&fn) {
    size_t Gn = groups.size();
#pragma omp parallel
    {
      std::vector<std::vector<size_t>> nb(Gn);
      for (auto &v : nb) v.reserve(100);
      for (auto *p : gs) {
        size_t pi = gidx(p);
#pragma omp for
        for (size_t i = 0; i < p->count; ++i) {
          for (auto &v : nb) v.clear();
          grid.neighbors(pi, i, [&](size_t ng, size_t ni) { nb[ng].push_back(ni); });
          fn(p, i, nb);
        }
      }
    }
  }

  // ---- procedures ----------------------------------------------------------
  void density_compute_density() {
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    for (auto *g : fl) {
      g->vf("position", 3); g->vf("density", 1); g->vf("mass", 1);
    }
    for (auto *g : bd) { g->vf("position", 3); g->vf("volume", 1); }
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density");
      T acc = 0;
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)]) acc += nm[j] * K.W(vsub(x[i], nx[j]));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)]) acc += (nV[j] * rho0) * K.W(vsub(x[i], nx[j]));
      }
      rho[i] = acc;
    });
  }

  // sesph.compute_density_and_pressure (schemes/sesph.hpp, generated from
  // share/schemes/sesph.prtcl): the density as density.compute_density,
  // then p = kappa max(0, rho / rho0 - 1), max as std::max({0, x})
  void sesph_compute_density_and_pressure() {
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    for (auto *g : fl) {
      g->vf("position", 3); g->vf("density", 1); g->vf("mass", 1); g->vf("pressure", 1);
    }
    for (auto *g : bd) { g->vf("position", 3); g->vf("volume", 1); }
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T rho0 = ur(*p, "rest_density"), kappa = ur(*p, "compressibility");
      T acc = 0;
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)]) acc += nm[j] * K.W(vsub(x[i], nx[j]));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)]) acc += (nV[j] * rho0) * K.W(vsub(x[i], nx[j]));
      }
      p->s1("density")[i] = acc;
      T t = acc / rho0 - T(1);
      p->s1("pressure")[i] = kappa * ((T(0) < t) ? t : T(0));
    });
  }

  // sesph.accumulate_acceleration: a -= m_j (p_i / rho_i^2 + p_j / rho_j^2)
  // gradW - (0.7 V_b rho0) (2 p_i / rho_i^2) gradW, into the existing a
  void sesph_accumulate_acceleration() {
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    for (auto *g : fl) {
      g->vf("position", 3); g->vf("acceleration", 3); g->vf("density", 1); g->vf("mass", 1);
      g->vf("pressure", 1);
    }
    for (auto *g : bd) { g->vf("position", 3); g->vf("volume", 1); }
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T *pr = p->s1("pressure");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density");
      V3<T> a = p->v3("acceleration")[i];
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        T *np = n->s1("pressure");
        T *nrho = n->s1("density");
        for (size_t j : nb[gidx(n)])
          a = vsub(a, vscale(nm[j] * ((pr[i] / (rho[i] * rho[i])) + (np[j] / (nrho[j] * nrho[j]))),
                             K.gradW(vsub(x[i], nx[j]))));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)])
          a = vsub(a, vscale(((T(0.7) * nV[j]) * rho0) * ((T(2) * pr[i]) / (rho[i] * rho[i])),
                             K.gradW(vsub(x[i], nx[j]))));
      }
      p->v3("acceleration")[i] = a;
    });
  }

  void aiast12_compute_volume() {
    auto bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    for (auto *g : bd) { g->vf("position", 3); g->vf("volume", 1); }
    foreach_with_neighbors(bd, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T acc = 0;
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        for (size_t j : nb[gidx(n)]) acc += K.W(vsub(x[i], nx[j]));
      }
      p->s1("volume")[i] = T(1) / acc;
    });
  }

  void gravity_initialize_acceleration() {
    V3<T> g = gv("gravity");
    for (auto *p : with_tag("dynamic")) {
      p->vf("position", 3);
      auto *a = p->v3("acceleration");
#pragma omp parallel for
      for (size_t i = 0; i < p->count; ++i) a[i] = g;
    }
  }

  void integrate_velocity_with_hard_fade() {
    T dt = gr("time_step"), t = gr("current_time"), fade = gr("fade_duration");
    for (auto *p : with_tag("dynamic")) {
      p->vf("position", 3);
      auto *v = p->v3("velocity");
      auto *a = p->v3("acceleration");
      T *tb = p->s1("time_of_birth");
#pragma omp parallel for schedule(static)
      for (size_t i = 0; i < p->count; ++i)
        v[i] = vadd(v[i], vscale(ustep(T(0), (t - tb[i]) - fade), vscale(dt, a[i])));
    }
  }

  void integrate_position() {
    T dt = gr("time_step");
    T ms = gr("maximum_speed");
    for (auto *p : with_tag("dynamic")) {
      auto *x = p->v3("position");
      auto *v = p->v3("velocity");
      p->vf("acceleration", 3); p->vf("time_of_birth", 1);
      T r = ms;
#pragma omp parallel for schedule(static) reduction(max : r)
      for (size_t i = 0; i < p->count; ++i) {
        x[i] = vadd(x[i], vscale(dt, v[i]));
        r = std::max(r, vnorm(v[i]));
      }
      ms = r;
    }
    gl("maximum_speed", 1)[0] = double(ms);
  }

  void iisph_fields() {
    for (auto *g : of_type("fluid")) {
      for (auto n : {"position", "velocity", "acceleration", "iisph_helper_c"}) g->vf(n, 3);
      for (auto n : {"density", "pressure", "mass", "iisph_source_term", "iisph_diagonal_element", "iisph_right_hand_side"})
        g->vf(n, 1);
    }
    for (auto *g : of_type("boundary")) { g->vf("position", 3); g->vf("volume", 1); }
  }

  void iisph_setup() {
    iisph_fields();
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    T h = K.h, dt = gr("time_step");
    (void)h;
    // pass 1: helper c
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T *m = p->s1("mass");
      (void)m;
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density");
      V3<T> c = {0, 0, 0};
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)])
          c = vsub(c, vscale(nm[j] / (rho[i] * rho[i]), K.gradW(vsub(x[i], nx[j]))));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)])
          c = vsub(c, vscale(((T(0.7) * T(2)) * rho0) * (nV[j] / (rho[i] * rho[i])), K.gradW(vsub(x[i], nx[j]))));
      }
      p->v3("iisph_helper_c")[i] = c;
    });
    // pass 2: p, s, AA; nprde counts the fluid particles
    int64_t nprde = 0;
    for (auto *p : fl) nprde += int64_t(p->count);
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      auto *v = p->v3("velocity");
      auto *c = p->v3("iisph_helper_c");
      T *m = p->s1("mass");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density");
      T s = 0, AA = 0;
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        auto *nv = n->v3("velocity");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)]) {
          s += nm[j] * vdot(vsub(v[i], nv[j]), K.gradW(vsub(x[i], nx[j])));
          AA += nm[j] * vdot(c[i], K.gradW(vsub(x[i], nx[j])));
          AA -= (nm[j] * (m[i] / (rho[i] * rho[i]))) * vnsq(K.gradW(vsub(x[i], nx[j])));
        }
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)]) {
          V3<T> zero = {0, 0, 0};
          s += (rho0 * nV[j]) * vdot(vsub(v[i], zero), K.gradW(vsub(x[i], nx[j])));
          AA += (rho0 * nV[j]) * vdot(c[i], K.gradW(vsub(x[i], nx[j])));
        }
      }
      p->s1("pressure")[i] = T(0);
      p->s1("iisph_source_term")[i] = (rho0 - rho[i]) - ((dt * (rho0 / rho[i])) * s);
      p->s1("iisph_diagonal_element")[i] = AA * ((dt * dt) * (rho0 / rho[i]));
    });
    gl("iisph_nprde", 1)[0] = double(nprde);
  }

  void iisph_iteration_pressure_acceleration() {
    iisph_fields();
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T *pr = p->s1("pressure");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density");
      V3<T> a = {0, 0, 0};
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        T *np = n->s1("pressure");
        T *nrho = n->s1("density");
        for (size_t j : nb[gidx(n)])
          a = vsub(a, vscale(nm[j] * ((pr[i] / (rho[i] * rho[i])) + (np[j] / (nrho[j] * nrho[j]))),
                             K.gradW(vsub(x[i], nx[j]))));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        for (size_t j : nb[gidx(n)])
          a = vsub(a, vscale(((T(0.7) * rho0) * nV[j]) * ((T(2) * pr[i]) / (rho[i] * rho[i])),
                             K.gradW(vsub(x[i], nx[j]))));
      }
      p->v3("acceleration")[i] = a;
    });
  }

  void iisph_iteration_pressure() {
    iisph_fields();
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    T dt = gr("time_step"), omega = gr("iisph_relaxation");
    T aprde0 = gr("iisph_aprde");
    // per-particle contributions to the density-error reduction
    std::vector<std::vector<T>> contrib(fl.size());
    for (size_t q = 0; q < fl.size(); ++q) contrib[q].assign(fl[q]->count, T(0));
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      auto *a = p->v3("acceleration");
      T *pr = p->s1("pressure");
      T *rho = p->s1("density");
      T *s = p->s1("iisph_source_term");
      T *AA = p->s1("iisph_diagonal_element");
      T rho0 = ur(*p, "rest_density");
      T Ap = 0;
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        auto *na = n->v3("acceleration");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)]) Ap += nm[j] * vdot(vsub(a[i], na[j]), K.gradW(vsub(x[i], nx[j])));
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        V3<T> zero = {0, 0, 0};
        for (size_t j : nb[gidx(n)]) Ap += (rho0 * nV[j]) * vdot(vsub(a[i], zero), K.gradW(vsub(x[i], nx[j])));
      }
      Ap *= (dt * dt) * (rho0 / rho[i]);
      p->s1("iisph_right_hand_side")[i] = Ap;
      T pn = std::max(T(0), pr[i] + ((omega * (s[i] - Ap)) * rcp0(AA[i], T(1e-9)))) * ustep(T(1e-9), std::abs(AA[i]));
      pr[i] = pn;
      size_t q = std::find(fl.begin(), fl.end(), p) - fl.begin();
      contrib[q][i] = ((Ap - s[i]) / rho0) * ustep(T(1e-9), pn);
    });
    if (fp64) {
      double acc = double(aprde0);
      for (auto &cv : contrib)
        for (T v : cv) acc += double(v);
      gl("iisph_aprde", 1)[0] = acc;
    } else {
      T acc = aprde0;
      for (auto &cv : contrib) {
        T r = 0;
        size_t n = cv.size();
#pragma omp parallel for reduction(+ : r)
        for (size_t i = 0; i < n; ++i) r += cv[i];
        acc += r;
      }
      gl("iisph_aprde", 1)[0] = double(acc);
    }
  }

  // ---- WKBB18 --------------------------------------------------------------
  void wkbb18_fields() {
    for (auto *g : of_type("fluid")) {
      for (auto n : {"position", "velocity", "acceleration", "wkbb18_velocity_delta"}) g->vf(n, 3);
      for (auto n : {"density", "mass", "time_of_birth"}) g->vf(n, 1);
      g->vf("wkbb18_system_diagonal", 9);
    }
    for (auto *g : of_type("boundary")) { g->vf("position", 3); g->vf("volume", 1); }
  }

  // gc: wkbb18_gc (share/schemes/wkbb18_gc.prtcl), every kernel gradient
  // premultiplied by the item's gradient correction L_i
  void wkbb18_compute_diagonal(bool gc = false) {
    wkbb18_fields();
    auto fl = of_type("fluid"), bd = of_type("boundary");
    if (gc)
      for (auto *g : fl) g->vf("gradient_correction", 9);
    Kernel<T> K(gr("smoothing_scale"));
    T h = K.h, dt = gr("time_step");
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto grad = [&](V3<T> const &xij) { return gc ? mvmul(p->m3("gradient_correction")[i], K.gradW(xij)) : K.gradW(xij); };
      auto *x = p->v3("position");
      T *m = p->s1("mass");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density"), mu = ur(*p, "dynamic_viscosity");
      M3<T> S;
      S.fill(T(0));
      auto acc_outer = [&](T coef, V3<T> const &g, V3<T> const &xij) {
        for (int c = 0; c < 3; ++c)
          for (int r = 0; r < 3; ++r) S[3 * c + r] += coef * (g[r] * xij[c]);
      };
      for (size_t j : nb[gidx(p)]) {
        V3<T> xij = vsub(x[i], x[j]);
        T coef = ((T(10) * (mu / rho[i])) * (m[j] / rho[j])) / (vnsq(xij) + ((T(0.01) * h) * h));
        acc_outer(coef, grad(xij), xij);
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        T nmu = ur(*n, "dynamic_viscosity");
        for (size_t j : nb[gidx(n)]) {
          V3<T> xij = vsub(x[i], nx[j]);
          T coef = ((T(10) * (nmu / rho[i])) * ((rho0 * nV[j]) / rho[i])) / (vnsq(xij) + ((T(0.01) * h) * h));
          acc_outer(coef, grad(xij), xij);
        }
      }
      M3<T> A;
      for (int c = 0; c < 3; ++c)
        for (int r = 0; r < 3; ++r) A[3 * c + r] = (r == c ? T(1) : T(0)) - dt * S[3 * c + r];
      p->m3("wkbb18_system_diagonal")[i] = minv(A);
    });
  }

  // correction.identity_gradient_correction / compute_gradient_correction
  // (share/schemes/correction.prtcl:14-43, schemes/correction.hpp:134-230):
  //   L_f = invert_pm(sum_{fluid neighbours} (m_j / rho_i) gradW(x_ij) (x_j - x_i)^T)
  void correction_identity() {
    for (auto *g : of_type("fluid")) {
      g->vf("gradient_correction", 9);
      auto *L = g->m3("gradient_correction");
      for (size_t i = 0; i < g->count; ++i) {
        L[i].fill(T(0));
        L[i][0] = L[i][4] = L[i][8] = T(1);
      }
    }
  }
  void correction_compute() {
    auto fl = of_type("fluid");
    for (auto *g : fl) {
      g->vf("position", 3);
      for (auto n : {"density", "mass"}) g->vf(n, 1);
      g->vf("gradient_correction", 9);
    }
    Kernel<T> K(gr("smoothing_scale"));
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      T *rho = p->s1("density");
      M3<T> Lf;
      Lf.fill(T(0));
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        T *nm = n->s1("mass");
        for (size_t j : nb[gidx(n)]) {
          V3<T> g = K.gradW(vsub(x[i], nx[j]));
          V3<T> d = vsub(nx[j], x[i]);
          T sc = nm[j] / rho[i];
          for (int c = 0; c < 3; ++c)
            for (int r = 0; r < 3; ++r) Lf[3 * c + r] = Lf[3 * c + r] + sc * (g[r] * d[c]);
        }
      }
      p->m3("gradient_correction")[i] = pinv3(Lf);
    });
  }

  // viscosity.accumulate_acceleration (share/schemes/viscosity.prtcl:31-66,
  // generated schemes/viscosity.hpp:171-240): explicit viscosity added to a,
  // over the neighbours of every fluid group, then of every boundary group
  // (boundary velocity zero)
  void viscosity_accumulate_acceleration() {
    for (auto *g : of_type("fluid")) {
      for (auto n : {"position", "velocity", "acceleration"}) g->vf(n, 3);
      for (auto n : {"density", "mass"}) g->vf(n, 1);
    }
    for (auto *g : of_type("boundary")) { g->vf("position", 3); g->vf("volume", 1); }
    auto fl = of_type("fluid"), bd = of_type("boundary");
    Kernel<T> K(gr("smoothing_scale"));
    T h = K.h;
    foreach_with_neighbors(fl, [&](Group<T> *p, size_t i, auto &nb) {
      auto *x = p->v3("position");
      auto *v = p->v3("velocity");
      auto *a = p->v3("acceleration");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density"), mu = ur(*p, "dynamic_viscosity");
      V3<T> ai = a[i];
      for (auto *n : fl) {
        auto *nx = n->v3("position");
        auto *nv = n->v3("velocity");
        T *nm = n->s1("mass");
        T *nrho = n->s1("density");
        for (size_t j : nb[gidx(n)]) {
          V3<T> xij = vsub(x[i], nx[j]);
          T coef = (((T(10) * (mu / rho[i])) * (nm[j] / nrho[j])) * vdot(vsub(v[i], nv[j]), xij)) /
                   (vnsq(xij) + ((T(0.01) * h) * h));
          ai = vadd(ai, vscale(coef, K.gradW(xij)));
        }
      }
      for (auto *n : bd) {
        auto *nx = n->v3("position");
        T *nV = n->s1("volume");
        T nmu = ur(*n, "dynamic_viscosity");
        for (size_t j : nb[gidx(n)]) {
          V3<T> xij = vsub(x[i], nx[j]);
          V3<T> zero{T(0), T(0), T(0)};
          T coef = (((T(10) * (nmu / rho[i])) * ((rho0 * nV[j]) / rho[i])) * vdot(vsub(v[i], zero), xij)) /
                   (vnsq(xij) + ((T(0.01) * h) * h));
          ai = vadd(ai, vscale(coef, K.gradW(xij)));
        }
      }
      a[i] = ai;
    });
  }

  // dot over a vector of 3-vectors: per item a0*b0 + (a1*b1 + a2*b2) in T,
  // accumulated in T (reference mode) or sequentially in double (FP64 mode)
  double cg_dot(std::vector<V3<T>> const &a, std::vector<V3<T>> const &b) const {
    size_t n = a.size();
    if (fp64) {
      double acc = 0;
      for (size_t i = 0; i < n; ++i) acc += double(vdot(a[i], b[i]));
      return acc;
    }
    T acc = 0;
#pragma omp parallel for schedule(static) reduction(+ : acc)
    for (size_t i = 0; i < n; ++i) acc += vdot(a[i], b[i]);
    return double(acc);
  }

  void wkbb18_accumulate_acceleration(bool gc = false) {
    wkbb18_fields();
    auto fl = of_type("fluid"), bd = of_type("boundary");
    if (gc)
      for (auto *g : fl) g->vf("gradient_correction", 9);
    Kernel<T> K(gr("smoothing_scale"));
    T h = K.h, dt = gr("time_step"), t = gr("current_time"), fade = gr("fade_duration");
    size_t Gn = groups.size();
    for (auto *p : fl) {
      size_t n = p->count;
      if (n == 0) { // solve() returns 0 for an empty group
        p->uf("wkbb18_iterations", 1)[0] = 0.0;
        continue;
      }
      auto *x = p->v3("position");
      auto *v = p->v3("velocity");
      T *m = p->s1("mass");
      T *rho = p->s1("density");
      T rho0 = ur(*p, "rest_density"), mu = ur(*p, "dynamic_viscosity");
      T tol = ur(*p, "wkbb18_maximum_error");
      int64_t max_k = int64_t(p->uf("wkbb18_maximum_iterations", 1)[0]);
      auto *sp = p->m3("wkbb18_system_diagonal");
      M3<T> const *Lc = gc ? p->m3("gradient_correction") : nullptr;
      size_t pi = gidx(p);
      std::vector<V3<T>> X(n), Y(n), Rr(n), P(n), Q(n), B(n);
      // system product: into = with - dt * a_f(with)  (wkbb18.hpp:339-396)
      auto system = [&](std::vector<V3<T>> &into, std::vector<V3<T>> const &with) {
#pragma omp parallel
        {
          std::vector<std::vector<size_t>> nb(Gn);
#pragma omp for
          for (size_t i = 0; i < n; ++i) {
            for (auto &vv : nb) vv.clear();
            grid.neighbors(pi, i, [&](size_t ng, size_t ni) { nb[ng].push_back(ni); });
            V3<T> af = {0, 0, 0};
            for (size_t j : nb[pi]) {
              V3<T> xij = vsub(x[i], x[j]);
              T coef = (((T(10) * (mu / rho[i])) * (m[j] / rho[j])) * vdot(vsub(with[i], with[j]), xij)) /
                       (vnsq(xij) + ((T(0.01) * h) * h));
              af = vadd(af, vscale(coef, Lc ? mvmul(Lc[i], K.gradW(xij)) : K.gradW(xij)));
            }
            for (auto *nn : bd) {
              auto *nx = nn->v3("position");
              T *nV = nn->s1("volume");
              T nmu = ur(*nn, "dynamic_viscosity");
              for (size_t j : nb[gidx(nn)]) {
                V3<T> xij = vsub(x[i], nx[j]);
                T coef = (((T(10) * (nmu / rho[i])) * ((rho0 * nV[j]) / rho[i])) * vdot(with[i], xij)) /
                         (vnsq(xij) + ((T(0.01) * h) * h));
                af = vadd(af, vscale(coef, Lc ? mvmul(Lc[i], K.gradW(xij)) : K.gradW(xij)));
              }
            }
            into[i] = vsub(with[i], vscale(dt, af));
          }
        }
      };
      // initial iterate and residual (cg_openmp.hpp:48-65); the right-hand
      // side's boundary term has v_b = 0, so b = v - dt * 0 = v exactly
      for (size_t i = 0; i < n; ++i) X[i] = v[i];
      system(Rr, X);
      for (size_t i = 0; i < n; ++i) {
        B[i] = vsub(v[i], vscale(dt, V3<T>{0, 0, 0}));
        Rr[i] = vsub(Rr[i], B[i]);
      }
      double b_nsq = cg_dot(B, B);
      double thr;
      if (fp64)
        thr = std::max(double(tol) * double(tol) * b_nsq, double(std::numeric_limits<T>::min()));
      else
        thr = double(std::max(T(tol * tol * T(b_nsq)), std::numeric_limits<T>::min()));
      for (size_t i = 0; i < n; ++i) {
        Y[i] = mvmul(sp[i], Rr[i]);
        P[i] = {-Y[i][0], -Y[i][1], -Y[i][2]};
      }
      double r_nsq = cg_dot(Rr, Rr);
      double next_rdy = cg_dot(Rr, Y);
      int64_t iter = 0;
      auto ok = [&](int64_t k, double cur) {
        if (k < 1) return true;
        if (k > max_k) return false;
        if (cur < thr) return false;
        return true;
      };
      for (iter = 0; ok(iter, r_nsq); ++iter) {
        double prev_rdy = next_rdy;
        system(Q, P);
        double pdq = cg_dot(P, Q);
        if (std::abs(pdq) < double(tol)) break;
        // FP64 mode: the scalar is formed in double and rounded once to T;
        // reference mode: T division of the T dot products
        T alpha = fp64 ? static_cast<T>(prev_rdy / pdq) : T(prev_rdy) / T(pdq);
        for (size_t i = 0; i < n; ++i) {
          X[i] = vadd(X[i], vscale(alpha, P[i]));
          Rr[i] = vadd(Rr[i], vscale(alpha, Q[i]));
        }
        r_nsq = cg_dot(Rr, Rr);
        for (size_t i = 0; i < n; ++i) Y[i] = mvmul(sp[i], Rr[i]);
        next_rdy = cg_dot(Rr, Y);
        if (std::abs(prev_rdy) < double(tol)) break;
        T beta = fp64 ? static_cast<T>(next_rdy / prev_rdy) : T(next_rdy) / T(prev_rdy);
        for (size_t i = 0; i < n; ++i) P[i] = vadd(V3<T>{-Y[i][0], -Y[i][1], -Y[i][2]}, vscale(beta, P[i]));
      }
      // apply (wkbb18.hpp:401-413)
      auto *vd = p->v3("wkbb18_velocity_delta");
      auto *a = p->v3("acceleration");
      T *tb = p->s1("time_of_birth");
      for (size_t i = 0; i < n; ++i) {
        vd[i] = vscale(ustep(T(0), (t - tb[i]) - fade), vsub(X[i], v[i]));
        a[i] = V3<T>{vd[i][0] / dt, vd[i][1] / dt, vd[i][2] / dt};
      }
      p->uf("wkbb18_iterations", 1)[0] = double(iter);
    }
  }

  // iisph.solve_pressure: the relaxed-Jacobi loop of the driver script
  // (share/scripts/prtcl-lua.example.lua:409-420) as one procedure: at least
  // two iterations, stop when aprde / nprde < iisph_maximum_density_error or
  // after iisph_maximum_iterations; writes iisph_iterations
  void iisph_solve_pressure() {
    int64_t maxit = int64_t(gl("iisph_maximum_iterations", 1)[0]);
    double eta = double(static_cast<T>(gl("iisph_maximum_density_error", 1)[0]));
    if (maxit <= 0) maxit = 100;
    if (!(eta > 0)) eta = double(static_cast<T>(1e-3));
    double nprde = gl("iisph_nprde", 1)[0];
    int64_t it = 0;
    if (nprde >= 1) {
      for (it = 1; it <= maxit; ++it) {
        gl("iisph_aprde", 1)[0] = 0.0;
        iisph_iteration_pressure_acceleration();
        iisph_iteration_pressure();
        double rel = gl("iisph_aprde", 1)[0] / nprde;
        if (it >= 2 && rel < eta) break;
      }
      if (it > maxit) it = maxit;
    }
    gl("iisph_iterations", 1)[0] = double(it);
  }

  void run(std::string const &scheme, std::string const &proc) override {
    if (scheme == "density" && proc == "compute_density") return density_compute_density();
    if (scheme == "sesph" && proc == "compute_density_and_pressure") return sesph_compute_density_and_pressure();
    if (scheme == "sesph" && proc == "accumulate_acceleration") return sesph_accumulate_acceleration();
    if (scheme == "aiast12" && proc == "compute_volume") return aiast12_compute_volume();
    if (scheme == "gravity" && proc == "initialize_acceleration") return gravity_initialize_acceleration();
    if (scheme == "symplectic_euler" && proc == "integrate_velocity_with_hard_fade")
      return integrate_velocity_with_hard_fade();
    if (scheme == "symplectic_euler" && proc == "integrate_position") return integrate_position();
    if (scheme == "iisph" && proc == "setup") return iisph_setup();
    if (scheme == "iisph" && proc == "iteration_pressure_acceleration") return iisph_iteration_pressure_acceleration();
    if (scheme == "iisph" && proc == "iteration_pressure") return iisph_iteration_pressure();
    if (scheme == "iisph" && proc == "solve_pressure") return iisph_solve_pressure();
    if (scheme == "wkbb18" && proc == "compute_diagonal") return wkbb18_compute_diagonal();
    if (scheme == "viscosity" && proc == "accumulate_acceleration") return viscosity_accumulate_acceleration();
    if (scheme == "wkbb18_gc" && proc == "compute_diagonal") return wkbb18_compute_diagonal(true);
    if (scheme == "wkbb18_gc" && proc == "accumulate_acceleration") return wkbb18_accumulate_acceleration(true);
    if (scheme == "correction" && proc == "identity_gradient_correction") return correction_identity();
    if (scheme == "correction" && proc == "compute_gradient_correction") return correction_compute();
    if (scheme == "wkbb18" && proc == "accumulate_acceleration") return wkbb18_accumulate_acceleration();
    throw std::runtime_error("procedure does not exist: " + scheme + "." + proc);
  }
};

} // namespace oracle

// ===========================================================================
// C ABI (ctypes)
// ===========================================================================

using oracle::SceneBase;

static thread_local std::string g_err;

#define ORACLE_TRY(body)                                                       \
  try {                                                                        \
    body;                                                                      \
    return 0;                                                                  \
  } catch (std::exception const &e) {                                          \
    g_err = e.what();                                                          \
    return -1;                                                                 \
  } catch (char const *e) {                                                    \
    g_err = e;                                                                 \
    return -1;                                                                 \
  }

extern "C" {

char const *oracle_last_error() { return g_err.c_str(); }

void *oracle_scene_new(int real_bytes, int fp64_reductions) {
  SceneBase *s = nullptr;
  if (real_bytes == 8) s = new oracle::Scene<double>();
  else s = new oracle::Scene<float>();
  s->fp64 = fp64_reductions != 0;
  return s;
}
void oracle_scene_free(void *s) { delete static_cast<SceneBase *>(s); }
// three-way Morton compare of n pairs of int32 triples (a[3 i..], b[3 i..])
void oracle_morton_compare_many(int32_t const *a, int32_t const *b, int64_t n, int8_t *out) {
  for (int64_t i = 0; i < n; ++i) {
    oracle::GI l{a[3 * i], a[3 * i + 1], a[3 * i + 2]}, r{b[3 * i], b[3 * i + 1], b[3 * i + 2]};
    out[i] = int8_t(oracle::morton_compare(l, r));
  }
}
// pseudo-inverses of n column-major 3x3 matrices (f32), for tests
void oracle_pinv3_many(float const *a, int64_t n, float *out) {
  for (int64_t k = 0; k < n; ++k) {
    oracle::M3<float> m;
    for (int e = 0; e < 9; ++e) m[e] = a[9 * k + e];
    oracle::M3<float> r = oracle::pinv3(m);
    for (int e = 0; e < 9; ++e) out[9 * k + e] = r[e];
  }
}
int oracle_set_threads(int n) {
  if (n > 0) omp_set_num_threads(n);
  return omp_get_max_threads();
}
int oracle_add_group(void *s, char const *name, char const *type) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->add_group(name, type));
}
int oracle_add_tag(void *s, char const *g, char const *tag) { ORACLE_TRY(static_cast<SceneBase *>(s)->add_tag(g, tag)); }
int oracle_resize(void *s, char const *g, int64_t n) { ORACLE_TRY(static_cast<SceneBase *>(s)->resize(g, size_t(n))); }
int oracle_group_index(void *s, char const *g) { return static_cast<SceneBase *>(s)->group_index(g); }
int oracle_set_varying(void *s, char const *g, char const *f, int ncomp, void const *data, int64_t n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->set_varying(g, f, ncomp, data, size_t(n)));
}
int oracle_get_varying(void *s, char const *g, char const *f, int ncomp, void *data, int64_t n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->get_varying(g, f, ncomp, data, size_t(n)));
}
int oracle_set_uniform(void *s, char const *g, char const *f, double const *v, int n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->set_uniform(g, f, v, n));
}
int oracle_get_uniform(void *s, char const *g, char const *f, double *v, int n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->get_uniform(g, f, v, n));
}
int oracle_set_global(void *s, char const *f, double const *v, int n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->set_global(f, v, n));
}
int oracle_get_global(void *s, char const *f, double *v, int n) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->get_global(f, v, n));
}
int oracle_set_radius(void *s, double r) { ORACLE_TRY(static_cast<SceneBase *>(s)->set_radius(r)); }
int oracle_nhood_update(void *s) { ORACLE_TRY(static_cast<SceneBase *>(s)->nhood_update()); }
int oracle_nhood_permute(void *s) { ORACLE_TRY(static_cast<SceneBase *>(s)->nhood_permute()); }
int oracle_run(void *s, char const *scheme, char const *proc) { ORACLE_TRY(static_cast<SceneBase *>(s)->run(scheme, proc)); }
int64_t oracle_grid_sorted_count(void *s) { return int64_t(static_cast<SceneBase *>(s)->grid_sorted_count()); }
int64_t oracle_grid_cell_count(void *s) { return int64_t(static_cast<SceneBase *>(s)->grid_cell_count()); }
int oracle_grid_dump(void *s, uint32_t *sorted, int32_t *gi, int32_t *range, int32_t *adj) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->grid_dump(sorted, gi, range, adj));
}
int64_t oracle_neighbors(void *s, int g, int64_t i, int64_t *counts, int64_t *out, int64_t cap) {
  try {
    return int64_t(static_cast<SceneBase *>(s)->neighbors(g, size_t(i), counts, out, size_t(cap)));
  } catch (std::exception const &e) {
    g_err = e.what();
    return -1;
  }
}
int oracle_neighbor_lists(void *s, int qg, int ng, int64_t *offsets, uint32_t *idx, int64_t cap) {
  ORACLE_TRY(static_cast<SceneBase *>(s)->neighbor_lists(qg, ng, offsets, idx, size_t(cap)));
}

// One dam-break step (share/scripts/prtcl-lua.example.lua:363-461):
// update (+ permute every `permute_every` steps), density, gravity,
// integrate velocity, IISPH setup and the relaxed-Jacobi loop
// (aprde := 0; pressure acceleration; pressure; stop when it >= 2 and
// aprde/nprde < eta, or at max_iters), integrate velocity, optional WKBB18
// (compute_diagonal, accumulate_acceleration, integrate velocity), integrate
// position.  stats[0] = Jacobi iterations, stats[1] = final aprde/nprde,
// stats[2] = PCG iterations (or -1).
int oracle_step(void *sp, int do_permute, int max_iters, double eta, int viscosity, double *stats) {
  auto *s = static_cast<SceneBase *>(sp);
  try {
    if (do_permute) s->nhood_permute();
    else s->nhood_update();
    s->run("density", "compute_density");
    s->run("gravity", "initialize_acceleration");
    s->run("symplectic_euler", "integrate_velocity_with_hard_fade");
    s->run("iisph", "setup");
    double nprde = 0, aprde = 0, rel = 0;
    s->get_global("iisph_nprde", &nprde, 1);
    int it = 0;
    if (nprde >= 1) {
      for (it = 1; it <= max_iters; ++it) {
        double zero = 0;
        s->set_global("iisph_aprde", &zero, 1);
        s->run("iisph", "iteration_pressure_acceleration");
        s->run("iisph", "iteration_pressure");
        s->get_global("iisph_aprde", &aprde, 1);
        rel = aprde / nprde;
        if (it >= 2 && rel < eta) break;
      }
      if (it > max_iters) it = max_iters;
    }
    s->run("symplectic_euler", "integrate_velocity_with_hard_fade");
    double pcg = -1;
    if (viscosity) {
      s->run("wkbb18", "compute_diagonal");
      s->run("wkbb18", "accumulate_acceleration");
      // first fluid group's iteration count (the scripts have one fluid group)
      s->run("symplectic_euler", "integrate_velocity_with_hard_fade");
    }
    s->run("symplectic_euler", "integrate_position");
    if (stats) {
      stats[0] = it;
      stats[1] = rel;
      stats[2] = pcg;
    }
    return 0;
  } catch (std::exception const &e) {
    g_err = e.what();
    return -1;
  }
}

} // extern "C"
