// prtcl_gpu.hpp -- header-only C++ facade over the C ABI (prtcl_gpu.h) that
// re-creates the reference's class names, so that driver code written
// against prtcl::Model / prtcl::Neighborhood / prtcl::SchemeBase
// (src/prtcl/data/model.hpp, src/prtcl/util/neighborhood.hpp:23-42,
// src/prtcl/schemes/scheme_base.hpp:18-105) compiles against the GPU library
// with the namespace changed to prtcl_gpu.  Errors throw, as the reference
// does (it throws `const char *` for unknown procedures / schemes; here
// std::out_of_range with the same message, std::runtime_error otherwise).
#ifndef PRTCL_GPU_HPP
#define PRTCL_GPU_HPP

#include "prtcl_gpu.h"

#include <algorithm>
#include <array>
#include <cstdint>
#include <memory>
#include <stdexcept>
#include <string>
#include <string_view>
#include <vector>

namespace prtcl_gpu {

inline void check(int rc) {
  if (rc == PRTCL_GPU_OK) return;
  if (rc == PRTCL_GPU_NOT_FOUND) throw std::out_of_range(prtcl_gpu_last_error());
  throw std::runtime_error(prtcl_gpu_last_error());
}

class Model;

// A group of the model (data/group.hpp).
class Group {
public:
  Group(prtcl_gpu_model *m, std::string name) : m_(m), name_(std::move(name)) {}
  std::string const &GetGroupName() const { return name_; }
  size_t GetItemCount() const {
    int64_t n = 0;
    check(prtcl_gpu_group_count(m_, name_.c_str(), &n));
    return size_t(n);
  }
  size_t GetGroupIndex() const {
    int32_t i = 0;
    check(prtcl_gpu_group_index(m_, name_.c_str(), &i));
    return size_t(i);
  }
  void AddTag(std::string_view tag) { check(prtcl_gpu_group_add_tag(m_, name_.c_str(), std::string(tag).c_str())); }
  void Resize(size_t n) { check(prtcl_gpu_group_resize(m_, name_.c_str(), int64_t(n))); }
  // varying fields: host layout of the reference (components contiguous per
  // item, matrices column-major)
  void AddVaryingField(std::string_view name, char const *ctype, std::vector<int32_t> extents) {
    check(prtcl_gpu_field_add(m_, name_.c_str(), std::string(name).c_str(), ctype, int32_t(extents.size()),
                              extents.data()));
  }
  void Upload(std::string_view field, void const *host, size_t count, void *stream = nullptr) {
    check(prtcl_gpu_field_upload(m_, name_.c_str(), std::string(field).c_str(), host, int64_t(count), stream));
  }
  void Download(std::string_view field, void *host, size_t count, void *stream = nullptr) const {
    check(prtcl_gpu_field_download(m_, name_.c_str(), std::string(field).c_str(), host, int64_t(count), stream));
  }
  void AddUniformField(std::string_view name, char const *ctype, std::vector<int32_t> extents) {
    check(prtcl_gpu_uniform_add(m_, name_.c_str(), std::string(name).c_str(), ctype, int32_t(extents.size()),
                                extents.data()));
  }
  void SetUniform(std::string_view name, void const *value) {
    check(prtcl_gpu_uniform_set(m_, name_.c_str(), std::string(name).c_str(), value));
  }
  void GetUniform(std::string_view name, void *value) const {
    check(prtcl_gpu_uniform_get(m_, name_.c_str(), std::string(name).c_str(), value));
  }
  // SaveVTK (util/save_vtk.cpp:57-128)
  void SaveVTK(std::string const &path) const {
    check(prtcl_gpu_group_save_vtk(m_, name_.c_str(), path.c_str()));
  }

private:
  prtcl_gpu_model *m_;
  std::string name_;
};

// data/model.hpp
class Model {
public:
  Model() { check(prtcl_gpu_model_create(&m_)); }
  ~Model() { prtcl_gpu_model_destroy(m_); }
  Model(Model const &) = delete;
  Model &operator=(Model const &) = delete;

  Group AddGroup(std::string_view name, std::string_view type) {
    check(prtcl_gpu_group_add(m_, std::string(name).c_str(), std::string(type).c_str()));
    return Group(m_, std::string(name));
  }
  Group GetGroup(std::string_view name) { return Group(m_, std::string(name)); }
  size_t GetGroupCount() const {
    int32_t n = 0;
    check(prtcl_gpu_model_group_count(m_, &n));
    return size_t(n);
  }
  void AddGlobalField(std::string_view name, char const *ctype, std::vector<int32_t> extents) {
    check(prtcl_gpu_global_add(m_, std::string(name).c_str(), ctype, int32_t(extents.size()), extents.data()));
  }
  void SetGlobal(std::string_view name, void const *value) {
    check(prtcl_gpu_global_set(m_, std::string(name).c_str(), value));
  }
  void GetGlobal(std::string_view name, void *value) const {
    check(prtcl_gpu_global_get(m_, std::string(name).c_str(), value));
  }
  void Synchronize() { check(prtcl_gpu_model_synchronize(m_, nullptr)); }
  // Model::Save / Model::Load in the reference's native binary archive format
  void Save(std::string const &path) { check(prtcl_gpu_model_save(m_, path.c_str())); }
  void Load(std::string const &path) { check(prtcl_gpu_model_load(m_, path.c_str())); }
  std::vector<std::string> GetGroupNames() const {
    int64_t need = 0;
    check(prtcl_gpu_model_group_names(m_, nullptr, 0, &need));
    std::string out(size_t(need), '\0');
    check(prtcl_gpu_model_group_names(m_, out.data(), need, &need));
    out.resize(out.size() ? out.size() - 1 : 0);
    std::vector<std::string> r;
    size_t a = 0;
    while (a < out.size()) {
      size_t b = out.find('\n', a);
      if (b == std::string::npos) b = out.size();
      if (b > a) r.push_back(out.substr(a, b - a));
      a = b + 1;
    }
    return r;
  }
  // device-loop statistics (prtcl_gpu_model_stats): Jacobi solves,
  // iterations, capped solves, largest aprde / nprde, PCG solves, iterations,
  // capped solves
  std::array<double, 7> Stats(bool reset = false) {
    std::array<double, 7> st{};
    check(prtcl_gpu_model_stats(m_, st.data(), 7, reset ? 1 : 0));
    return st;
  }
  prtcl_gpu_model *handle() const { return m_; }

private:
  prtcl_gpu_model *m_ = nullptr;
};

// util/neighborhood.hpp:23-42
class Neighborhood {
public:
  Neighborhood() { check(prtcl_gpu_nhood_create(&n_)); }
  ~Neighborhood() { prtcl_gpu_nhood_destroy(n_); }
  Neighborhood(Neighborhood const &) = delete;
  Neighborhood &operator=(Neighborhood const &) = delete;

  void SetRadius(double radius) { check(prtcl_gpu_nhood_set_radius(n_, radius)); }
  void Load(Model const &model) {
    model_ = model.handle();
    check(prtcl_gpu_nhood_load(n_, model_));
  }
  void Update() { check(prtcl_gpu_nhood_update(n_, nullptr)); }
  void Permute(Model &model) { check(prtcl_gpu_nhood_permute(n_, model.handle(), nullptr)); }
  // neighbors[g] receives the raw indices of the neighbours in group g, in
  // the reference's traversal order
  void CopyNeighbors(size_t g, size_t i, std::vector<std::vector<size_t>> &neighbors) const {
    int32_t groups = 0;
    check(prtcl_gpu_model_group_count(model_, &groups));
    std::vector<int64_t> counts(static_cast<size_t>(groups)), idx(4096);
    int64_t total = 0;
    check(prtcl_gpu_nhood_copy_neighbors(n_, int32_t(g), int64_t(i), counts.data(), idx.data(), int64_t(idx.size()),
                                         &total));
    if (total > int64_t(idx.size())) {
      idx.resize(size_t(total));
      check(prtcl_gpu_nhood_copy_neighbors(n_, int32_t(g), int64_t(i), counts.data(), idx.data(),
                                           int64_t(idx.size()), &total));
    }
    neighbors.resize(size_t(groups));
    size_t o = 0;
    for (size_t q = 0; q < size_t(groups); ++q)
      for (int64_t k = 0; k < counts[q]; ++k) neighbors[q].push_back(size_t(idx[o++]));
  }
  prtcl_gpu_nhood *handle() const { return n_; }

private:
  prtcl_gpu_nhood *n_ = nullptr;
  prtcl_gpu_model *model_ = nullptr;
};

// schemes/scheme_base.hpp:18-64
class SchemeBase {
public:
  explicit SchemeBase(prtcl_gpu_scheme *s) : s_(s) {}
  ~SchemeBase() { prtcl_gpu_scheme_destroy(s_); }
  SchemeBase(SchemeBase const &) = delete;
  SchemeBase &operator=(SchemeBase const &) = delete;

  std::string GetFullName() const { return read(prtcl_gpu_scheme_full_name); }
  void Load(Model &model) { check(prtcl_gpu_scheme_load(s_, model.handle())); }
  void RunProcedure(std::string_view name, Neighborhood const &nhood, void *stream = nullptr) {
    check(prtcl_gpu_scheme_run(s_, std::string(name).c_str(), nhood.handle(), stream));
  }
  std::vector<std::string> GetProcedureNames() const { return split(read(prtcl_gpu_scheme_procedure_names)); }
  std::string GetPrtclSourceCode() const { return read(prtcl_gpu_scheme_source); }

  static std::vector<std::string> split(std::string const &s) {
    std::vector<std::string> r;
    size_t a = 0;
    while (a <= s.size()) {
      size_t b = s.find('\n', a);
      if (b == std::string::npos) b = s.size();
      if (b > a) r.push_back(s.substr(a, b - a));
      a = b + 1;
    }
    return r;
  }

private:
  template <class F> std::string read(F f) const {
    int64_t need = 0;
    check(f(s_, nullptr, 0, &need));
    std::string out(size_t(need), '\0');
    check(f(s_, out.data(), need, &need));
    out.resize(out.size() ? out.size() - 1 : 0);
    return out;
  }
  prtcl_gpu_scheme *s_;
};

// schemes/scheme_base.hpp:66-105
class SchemeRegistry {
public:
  static std::unique_ptr<SchemeBase> NewScheme(std::string_view full_name) {
    prtcl_gpu_scheme *s = nullptr;
    check(prtcl_gpu_scheme_new(std::string(full_name).c_str(), &s));
    return std::make_unique<SchemeBase>(s);
  }
  static std::vector<std::string> GetSchemeNames() {
    int64_t need = 0;
    check(prtcl_gpu_registry_scheme_names(nullptr, 0, &need));
    std::string out(size_t(need), '\0');
    check(prtcl_gpu_registry_scheme_names(out.data(), need, &need));
    out.resize(out.size() ? out.size() - 1 : 0);
    return SchemeBase::split(out);
  }
};

inline SchemeRegistry &GetSchemeRegistry() {
  static SchemeRegistry r;
  return r;
}

// Batched scenes (prtcl_gpu_batch_*): no reference counterpart; the
// reference runs one scene per process.
class Batch {
public:
  explicit Batch(prtcl_gpu_batch_params const &p) { check(prtcl_gpu_batch_create(&p, &b_)); }
  ~Batch() { prtcl_gpu_batch_destroy(b_); }
  Batch(Batch const &) = delete;
  Batch &operator=(Batch const &) = delete;

  int64_t AddScene(std::vector<float> const &fluid_xyz, std::vector<float> const &boundary_xyz) {
    int64_t id = 0;
    check(prtcl_gpu_batch_add_scene(b_, fluid_xyz.data(), int64_t(fluid_xyz.size() / 3), boundary_xyz.data(),
                                    int64_t(boundary_xyz.size() / 3), &id));
    return id;
  }
  void RemoveScene(int64_t id) { check(prtcl_gpu_batch_remove_scene(b_, id)); }
  void Step(int32_t steps = 1) { check(prtcl_gpu_batch_step(b_, steps)); }
  void Synchronize() { check(prtcl_gpu_batch_synchronize(b_)); }
  prtcl_gpu_scene_info Info(int64_t id) {
    prtcl_gpu_scene_info s{};
    check(prtcl_gpu_batch_scene_info(b_, id, &s));
    return s;
  }
  std::vector<float> Positions(int64_t id) {
    prtcl_gpu_scene_info s = Info(id);
    std::vector<float> x(size_t(s.fluid) * 3);
    check(prtcl_gpu_batch_download(b_, id, "position", x.data(), s.fluid));
    return x;
  }
  prtcl_gpu_batch *handle() { return b_; }

private:
  prtcl_gpu_batch *b_ = nullptr;
};

// The serving loop (prtcl_gpu_server_*) over a batch of its own.
class Server {
public:
  struct Result {
    prtcl_gpu_request_result r;
    std::vector<float> positions; // empty unless keep_results
  };
  Server(prtcl_gpu_batch_params const &batch, prtcl_gpu_server_params const &p) : keep_(p.keep_results != 0) {
    check(prtcl_gpu_server_create(&batch, &p, &s_));
  }
  ~Server() { prtcl_gpu_server_destroy(s_); }
  Server(Server const &) = delete;
  Server &operator=(Server const &) = delete;

  void Submit(int64_t request_id, double arrival, std::vector<float> const &fluid_xyz,
              std::vector<float> const &boundary_xyz, int64_t steps) {
    check(prtcl_gpu_server_submit(s_, request_id, arrival, fluid_xyz.data(), int64_t(fluid_xyz.size() / 3),
                                  boundary_xyz.data(), int64_t(boundary_xyz.size() / 3), steps));
    max_fluid_ = std::max<int64_t>(max_fluid_, int64_t(fluid_xyz.size() / 3));
  }
  // one turn; false when nothing was resident
  bool Turn() {
    int32_t stepped = 0;
    check(prtcl_gpu_server_turn(s_, &stepped));
    return stepped != 0;
  }
  // retire a queued or resident request as cancelled; false if none has the id
  bool Cancel(int64_t request_id) {
    int32_t found = 0;
    check(prtcl_gpu_server_cancel(s_, request_id, &found));
    return found != 0;
  }
  prtcl_gpu_server_status Status() {
    prtcl_gpu_server_status st{};
    check(prtcl_gpu_server_status_get(s_, &st));
    return st;
  }
  // the retired requests not yet read, oldest first
  std::vector<Result> TakeResults() {
    std::vector<Result> out;
    std::vector<float> buf(keep_ ? size_t(max_fluid_) * 3 : 0);
    for (;;) {
      Result r{};
      int32_t has = 0;
      check(prtcl_gpu_server_next_result(s_, &r.r, keep_ ? buf.data() : nullptr, keep_ ? max_fluid_ : 0, &has));
      if (!has) break;
      if (keep_) r.positions.assign(buf.begin(), buf.begin() + size_t(r.r.fluid) * 3);
      out.push_back(std::move(r));
    }
    return out;
  }

private:
  prtcl_gpu_server *s_ = nullptr;
  bool keep_;
  int64_t max_fluid_ = 0;
};

} // namespace prtcl_gpu

#endif // PRTCL_GPU_HPP
