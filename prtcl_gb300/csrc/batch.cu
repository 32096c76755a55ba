// Batched scenes (see batch.hpp).
#include "batch.hpp"

#include <algorithm>
#include <cstring>
#include <set>

namespace prtcl_gpu {

namespace {
constexpr uint32_t kNoSrc = 0xFFFFFFFFu;
char const *kSchemes[] = {"density", "gravity", "symplectic_euler", "iisph", "wkbb18", "aiast12"};
std::string full(char const *n) { return std::string("prtcl::schemes::") + n + "[T=f32, N=3, K=Cubic Spline]"; }
} // namespace

Batch::Batch(prtcl_gpu_batch_params const &p) : p_(p) {
  if (!(p.smoothing_scale > 0.0) || !(p.time_step > 0.0) || !(p.rest_density > 0.0))
    throw Error("batch: smoothing_scale, time_step and rest_density must be positive");
  if (p.permute_every < 1) throw Error("batch: permute_every must be >= 1");
  if (p.max_iterations < 1) throw Error("batch: max_iterations must be >= 1");
  b_ = &m_.add_group("b", "boundary");
  f_ = &m_.add_group("f", "fluid");
  f_->tags.insert("dynamic");
  std::unique_ptr<Scheme> *dst[] = {&density_, &gravity_, &euler_, &iisph_, &wkbb18_, &aiast12_};
  for (int k = 0; k < 6; ++k) {
    *dst[k] = new_scheme(full(kSchemes[k]));
    (*dst[k])->load(m_);
  }
  // globals and uniforms of the set-up (share/scripts/prtcl-lua.example.lua:
  // 122-186, 288-316): f32 values; particles are born one second before they
  // are added, with no fade-in, so the hard fade of the velocity integration
  // is open from the scene's first step
  float h = float(p.smoothing_scale), dt = float(p.time_step), rho0 = float(p.rest_density);
  float g[3] = {float(p.gravity[0]), float(p.gravity[1]), float(p.gravity[2])};
  float omega = float(p.relaxation), eta = float(p.max_density_error), zero = 0.0f;
  int32_t maxit = p.max_iterations, izero = 0;
  set_global("smoothing_scale", &h);
  set_global("time_step", &dt);
  set_global("gravity", g);
  set_global("iisph_relaxation", &omega);
  set_global("fade_duration", &zero);
  set_global("current_time", &zero);
  set_global("maximum_speed", &zero);
  set_global("iisph_maximum_iterations", &maxit);
  set_global("iisph_maximum_density_error", &eta);
  set_global("iisph_iterations", &izero);
  float mu = float(p.dynamic_viscosity), mub = float(p.boundary_dynamic_viscosity), tol = float(p.pcg_max_error);
  int32_t pmax = p.pcg_max_iterations;
  cudaStream_t s = m_.stream();
  m_.small_set(f_->uniform.at("rest_density"), &rho0, s);
  m_.small_set(f_->uniform.at("dynamic_viscosity"), &mu, s);
  m_.small_set(f_->uniform.at("wkbb18_maximum_error"), &tol, s);
  m_.small_set(f_->uniform.at("wkbb18_maximum_iterations"), &pmax, s);
  m_.small_set(b_->uniform.at("dynamic_viscosity"), &mub, s);
  m_.seg = std::make_unique<Segments>();
  m_.seg->set_slots(0, s);
  nh_.load(m_);
  nh_.set_radius(2.0 * double(h));
  PG_CUDA(cudaStreamSynchronize(s));
}

Batch::~Batch() { cudaStreamSynchronize(m_.stream()); }

void Batch::set_global(char const *name, void const *value) {
  SmallField *f = m_.find_global(name);
  if (!f) throw Error(std::string("batch: global missing: ") + name);
  m_.small_set(*f, value, m_.stream());
}

void Batch::run(Scheme &s, char const *proc) { s.run(proc, nh_, m_.stream()); }

int64_t Batch::add(float const *xf, size_t nf, float const *xb, size_t nb) {
  if (nf && !xf) throw Error("batch: fluid positions missing");
  if (nb && !xb) throw Error("batch: boundary positions missing");
  Scene sc;
  sc.id = next_id_++;
  sc.nf = nf;
  sc.nb = nb;
  sc.xf.assign(xf, xf + 3 * nf);
  sc.xb.assign(xb, xb + 3 * nb);
  scenes_.push_back(std::move(sc));
  dirty_ = true;
  return scenes_.back().id;
}

Batch::Scene &Batch::find(int64_t id) {
  for (auto &sc : scenes_)
    if (sc.id == id && std::find(removed_.begin(), removed_.end(), id) == removed_.end()) return sc;
  throw Error("batch: no scene " + std::to_string(id));
}

void Batch::remove(int64_t id) {
  Scene &sc = find(id);
  if (sc.fresh) {
    scenes_.erase(std::find_if(scenes_.begin(), scenes_.end(), [&](Scene const &x) { return x.id == id; }));
    return;
  }
  removed_.push_back(id);
  dirty_ = true;
}

size_t Batch::scene_count() const { return scenes_.size() - removed_.size(); }

// Applies pending additions and removals: remaps both groups into the new
// slot ranges, uploads the new scenes and sets them up.
void Batch::commit() {
  if (!dirty_) return;
  cudaStream_t s = m_.stream();
  // 1. survivors keep their slots; new scenes take the lowest free ones
  std::vector<Scene> keep;
  std::set<uint32_t> used;
  for (auto &sc : scenes_) {
    if (std::find(removed_.begin(), removed_.end(), sc.id) != removed_.end()) continue;
    if (!sc.fresh) used.insert(sc.slot);
    keep.push_back(std::move(sc));
  }
  uint32_t next = 0;
  for (auto &sc : keep)
    if (sc.fresh) {
      while (used.count(next)) ++next;
      sc.slot = next;
      used.insert(next);
    }
  uint32_t slots = used.empty() ? 0u : *used.rbegin() + 1u;
  if (slots > 65536) throw Error("batch: at most 65536 scenes");
  std::sort(keep.begin(), keep.end(), [](Scene const &a, Scene const &b) { return a.slot < b.slot; });
  // 2. per-slot counts and the remap of each group (new index -> old index)
  std::vector<uint32_t> fcount(slots, 0), bcount(slots, 0);
  std::vector<uint32_t> fmap, bmap;
  for (auto &sc : keep) {
    fcount[sc.slot] = uint32_t(sc.nf);
    bcount[sc.slot] = uint32_t(sc.nb);
    for (size_t k = 0; k < sc.nf; ++k) fmap.push_back(sc.fresh ? kNoSrc : uint32_t(fstart_[sc.slot] + k));
    for (size_t k = 0; k < sc.nb; ++k) bmap.push_back(sc.fresh ? kNoSrc : uint32_t(bstart_[sc.slot] + k));
  }
  auto remap = [&](Group *g, std::vector<uint32_t> const &map) {
    uint32_t *d = nullptr;
    if (!map.empty()) {
      PG_CUDA(cudaMallocAsync(&d, map.size() * 4, s));
      PG_CUDA(cudaMemcpyAsync(d, map.data(), map.size() * 4, cudaMemcpyHostToDevice, s));
    }
    g->remap(d, map.size(), s);
    if (d) PG_CUDA(cudaFreeAsync(d, s));
  };
  remap(f_, fmap);
  remap(b_, bmap);
  // 3. segments (slot state of survivors kept; new scenes start from zero)
  Segments &S = *m_.seg;
  S.set_slots(slots, s);
  for (auto &sc : keep)
    if (sc.fresh) S.reset_slot(sc.slot, s);
  S.assign(b_, bcount, s);
  S.assign(f_, fcount, s);
  std::vector<int> np(std::max<uint32_t>(slots, 1), 0);
  for (uint32_t k = 0; k < slots; ++k) np[k] = int(fcount[k]);
  PG_CUDA(cudaMemcpyAsync(S.nprde, np.data(), np.size() * sizeof(int), cudaMemcpyHostToDevice, s));
  // groups by index: "b" 0, "f" 1
  nh_.set_segments({S.find(b_)->seg, S.find(f_)->seg}, slots);
  fstart_ = S.find(f_)->start;
  bstart_ = S.find(b_)->start;
  // 4. upload the new scenes (velocity, acceleration, density, ... are zero)
  float h = float(p_.smoothing_scale), rho0 = float(p_.rest_density);
  float mass = float(double(h) * double(h) * double(h) * double(rho0));
  float tb = float(t_) - 1.0f;
  std::vector<uint8_t> due(std::max<uint32_t>(slots, 1), 0);
  bool any_fresh = false;
  VaryingField *fx = f_->find_varying("position"), *fm = f_->find_varying("mass");
  VaryingField *ft = f_->find_varying("time_of_birth"), *bx = b_->find_varying("position");
  for (auto &sc : keep) {
    if (!sc.fresh) continue;
    any_fresh = true;
    due[sc.slot] = 1;
    std::vector<float> m(sc.nf, mass), t(sc.nf, tb);
    upload_varying_range(*fx, fstart_[sc.slot], sc.xf.data(), sc.nf, s);
    upload_varying_range(*fm, fstart_[sc.slot], m.data(), sc.nf, s);
    upload_varying_range(*ft, fstart_[sc.slot], t.data(), sc.nf, s);
    upload_varying_range(*bx, bstart_[sc.slot], sc.xb.data(), sc.nb, s);
    // the host vectors above must outlive their copies
    PG_CUDA(cudaStreamSynchronize(s));
  }
  scenes_ = std::move(keep);
  removed_.clear();
  slots_ = slots;
  dirty_ = false;
  // 5. set-up of the new scenes: update, permute (new slots only), volumes
  if (any_fresh) {
    nh_.update(s);
    PG_CUDA(cudaMemcpyAsync(S.due, due.data(), due.size(), cudaMemcpyHostToDevice, s));
    nh_.permute_segments(m_, S.due, s);
    run(*aiast12_, "compute_volume");
    PG_CUDA(cudaStreamSynchronize(s));
  }
  for (auto &sc : scenes_) {
    if (!sc.fresh) continue;
    sc.fresh = false;
    sc.since_permute = 0;
    sc.xf.clear();
    sc.xf.shrink_to_fit();
    sc.xb.clear();
    sc.xb.shrink_to_fit();
  }
}

// One step of every scene (share/scripts/prtcl-lua.example.lua:363-461, with
// the device-side Jacobi loop), each scene permuted on its own schedule.
void Batch::step(int k) {
  commit();
  cudaStream_t s = m_.stream();
  Segments &S = *m_.seg;
  bool visc = p_.viscosity != 0;
  std::vector<uint8_t> due(std::max<uint32_t>(slots_, 1), 0);
  for (int it = 0; it < k; ++it) {
    if (scenes_.empty()) {
      t_ += double(float(p_.time_step));
      continue;
    }
    float tf = float(t_);
    m_.small_set_async(*m_.find_global("current_time"), &tf, s);
    nh_.update(s);
    bool any = false;
    std::fill(due.begin(), due.end(), uint8_t(0));
    for (auto &sc : scenes_)
      if (++sc.since_permute >= p_.permute_every) {
        due[sc.slot] = 1;
        sc.since_permute = 0;
        any = true;
      }
    if (any) {
      // pageable source: the call returns once the bytes are staged
      PG_CUDA(cudaMemcpyAsync(S.due, due.data(), due.size(), cudaMemcpyHostToDevice, s));
      nh_.permute_segments(m_, S.due, s);
    }
    run(*density_, "compute_density");
    run(*gravity_, "initialize_acceleration");
    run(*euler_, "integrate_velocity_with_hard_fade");
    run(*iisph_, "setup");
    run(*iisph_, "solve_pressure");
    run(*euler_, "integrate_velocity_with_hard_fade");
    if (visc) {
      run(*wkbb18_, "compute_diagonal");
      run(*wkbb18_, "accumulate_acceleration");
      run(*euler_, "integrate_velocity_with_hard_fade");
    }
    run(*euler_, "integrate_position");
    t_ += double(float(p_.time_step));
    for (auto &sc : scenes_) ++sc.steps;
  }
}

void Batch::synchronize() {
  commit();
  PG_CUDA(cudaStreamSynchronize(m_.stream()));
}

prtcl_gpu_scene_info Batch::info(int64_t id) {
  commit();
  Scene &sc = find(id);
  cudaStream_t s = m_.stream();
  Segments &S = *m_.seg;
  int st[8];
  double sv[8];
  int it = 0;
  PG_CUDA(cudaMemcpyAsync(st, S.stat + size_t(sc.slot) * 8, sizeof st, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(sv, S.stats + size_t(sc.slot) * 8, sizeof sv, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaMemcpyAsync(&it, S.iters + sc.slot, sizeof it, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  prtcl_gpu_scene_info r{};
  r.fluid = int64_t(sc.nf);
  r.boundary = int64_t(sc.nb);
  r.steps = sc.steps;
  r.slot = int32_t(sc.slot);
  r.last_jacobi_iterations = sc.steps ? st[4] : 0;
  r.last_pcg_iterations = (sc.steps && p_.viscosity) ? it : 0;
  r.last_relative_density_error = sv[7];
  r.max_relative_density_error = sv[3];
  r.jacobi_solves = sv[0];
  r.jacobi_iterations = sv[1];
  r.jacobi_capped = sv[2];
  r.pcg_solves = sv[4];
  r.pcg_iterations = sv[5];
  r.pcg_capped = sv[6];
  return r;
}

void Batch::download(int64_t id, std::string const &field, void *host, size_t n) {
  commit();
  Scene &sc = find(id);
  if (n != sc.nf)
    throw Error("batch download: item count " + std::to_string(n) + " != scene fluid count " + std::to_string(sc.nf));
  VaryingField *f = f_->find_varying(field);
  if (!f) throw Error("field does not exist: f." + field);
  download_varying_range(*f, fstart_[sc.slot], host, n, m_.stream());
}

void Batch::particles(int64_t &nf, int64_t &nb) {
  commit();
  nf = int64_t(f_->count);
  nb = int64_t(b_->count);
}

size_t Batch::device_bytes() {
  commit();
  return m_.device_bytes() + nh_.device_bytes();
}

} // namespace prtcl_gpu
