// Serving loop (server.hpp).
#include "batch.hpp"
#include "server.hpp"

#include <algorithm>
#include <cmath>
#include <limits>
#include <string>

namespace prtcl_gpu {

namespace {

class DeviceServeBatch : public ServeBatch {
public:
  explicit DeviceServeBatch(prtcl_gpu_batch_params const &p) : b_(p) {}
  int64_t add(float const *xf, size_t nf, float const *xb, size_t nb) override { return b_.add(xf, nf, xb, nb); }
  void remove(int64_t id) override { b_.remove(id); }
  void step(int k) override { b_.step(k); }
  void synchronize() override { b_.synchronize(); }
  size_t device_bytes() override { return b_.device_bytes(); }
  prtcl_gpu_scene_info info(int64_t id) override { return b_.info(id); }
  void download_positions(int64_t id, float *host, size_t n) override { b_.download(id, "position", host, n); }

private:
  Batch b_;
};

class CallbackServeBatch : public ServeBatch {
public:
  CallbackServeBatch(prtcl_gpu_server_batch_ops const &ops, void *user) : o_(ops), u_(user) {
    if (!o_.add_scene || !o_.remove_scene || !o_.step || !o_.device_bytes || !o_.scene_info)
      throw Error("server batch operations: add_scene, remove_scene, step, device_bytes and scene_info are required");
  }
  int64_t add(float const *xf, size_t nf, float const *xb, size_t nb) override {
    int64_t id = 0;
    ok(o_.add_scene(u_, xf, int64_t(nf), xb, int64_t(nb), &id), "add_scene");
    return id;
  }
  void remove(int64_t id) override { ok(o_.remove_scene(u_, id), "remove_scene"); }
  void step(int k) override { ok(o_.step(u_, k), "step"); }
  void synchronize() override {
    if (o_.synchronize) ok(o_.synchronize(u_), "synchronize");
  }
  size_t device_bytes() override {
    int64_t v = 0;
    ok(o_.device_bytes(u_, &v), "device_bytes");
    return size_t(std::max<int64_t>(v, 0));
  }
  prtcl_gpu_scene_info info(int64_t id) override {
    prtcl_gpu_scene_info s{};
    ok(o_.scene_info(u_, id, &s), "scene_info");
    return s;
  }
  void download_positions(int64_t id, float *host, size_t n) override {
    if (!o_.download_positions) throw Error("server batch operations: download_positions is required to keep results");
    ok(o_.download_positions(u_, id, host, int64_t(n)), "download_positions");
  }

private:
  static void ok(int rc, char const *what) {
    if (rc != 0) throw Error(std::string("server batch operation failed: ") + what);
  }
  prtcl_gpu_server_batch_ops o_;
  void *u_;
};

} // namespace

std::unique_ptr<ServeBatch> device_serve_batch(prtcl_gpu_batch_params const &p) {
  return std::make_unique<DeviceServeBatch>(p);
}
std::unique_ptr<ServeBatch> callback_serve_batch(prtcl_gpu_server_batch_ops const &ops, void *user) {
  return std::make_unique<CallbackServeBatch>(ops, user);
}

Server::Server(std::unique_ptr<ServeBatch> batch, prtcl_gpu_server_params const &p)
    : b_(std::move(batch)), p_(p), t0_(std::chrono::steady_clock::now()) {
  if (p_.max_scenes < 1) throw Error("server: max_scenes must be >= 1");
  if (!(p_.budget_bytes >= 0.0)) throw Error("server: budget_bytes must be >= 0");
  if (!(p_.bytes_per_particle >= 0.0)) throw Error("server: bytes_per_particle must be >= 0");
  bpp_ = p_.bytes_per_particle;
}

double Server::now() const {
  if (p_.clock) return p_.clock(p_.clock_user);
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0_).count();
}

void Server::submit(int64_t rid, double arrival, float const *xf, size_t nf, float const *xb, size_t nb,
                    int64_t steps) {
  if (steps < 1) throw Error("server: a request needs at least one step");
  if (!std::isfinite(arrival)) throw Error("server: arrival time is not finite");
  if ((nf && !xf) || (nb && !xb)) throw Error("server: particle positions are null");
  double need = double(nf + nb) * bpp_;
  if (need > p_.budget_bytes)
    throw Error("server: the request needs an estimated " + std::to_string(int64_t(need)) +
                " device bytes, more than the budget of " + std::to_string(int64_t(p_.budget_bytes)));
  Request r;
  r.rid = rid;
  r.arrival = arrival;
  r.steps = steps;
  r.nf = nf;
  r.nb = nb;
  r.xf.assign(xf, xf + 3 * nf);
  r.xb.assign(xb, xb + 3 * nb);
  // after every pending request that arrives no later (submission order on ties)
  auto at = std::upper_bound(pending_.begin(), pending_.end(), arrival,
                             [](double a, Request const &q) { return a < q.arrival; });
  pending_.insert(at, std::move(r));
}

Server::Result Server::result_of(Request const &x, int32_t status, bool resident) {
  Result res;
  res.r.request_id = x.rid;
  res.r.fluid = int64_t(x.nf);
  res.r.boundary = int64_t(x.nb);
  res.r.steps = x.done;
  res.r.arrival = x.arrival;
  res.r.admitted = resident ? x.admitted : -1.0;
  res.r.status = status;
  if (resident) {
    try {
      res.r.info = b_->info(x.sid);
    } catch (std::exception const &) {
      res.r.info = prtcl_gpu_scene_info{};
      if (res.r.status == PRTCL_GPU_REQUEST_DONE) res.r.status = PRTCL_GPU_REQUEST_FAILED;
    }
  }
  res.r.finished = now();
  return res;
}

void Server::drop_scene(int64_t sid) {
  try {
    b_->remove(sid);
  } catch (std::exception const &) {
    orphans_.push_back(sid);
  }
}

bool Server::cancel(int64_t rid) {
  for (auto it = pending_.begin(); it != pending_.end(); ++it)
    if (it->rid == rid) {
      results_.push_back(result_of(*it, PRTCL_GPU_REQUEST_CANCELLED, false));
      pending_.erase(it);
      return true;
    }
  for (auto it = running_.begin(); it != running_.end(); ++it)
    if (it->rid == rid) {
      results_.push_back(result_of(*it, PRTCL_GPU_REQUEST_CANCELLED, true));
      drop_scene(it->sid);
      running_.erase(it);
      held_ = running_.empty() ? 0.0 : double(b_->device_bytes());
      return true;
    }
  return false;
}

bool Server::turn() {
  // 0. scenes whose removal failed earlier
  for (size_t k = 0; k < orphans_.size();) {
    try {
      b_->remove(orphans_[k]);
      orphans_.erase(orphans_.begin() + std::ptrdiff_t(k));
    } catch (std::exception const &) {
      ++k;
    }
  }
  double t = now();
  // 1. admissions, in arrival order, within the slots and the budget
  while (!pending_.empty() && pending_.front().arrival <= t && running_.size() < size_t(p_.max_scenes)) {
    Request &q = pending_.front();
    double need = double(q.nf + q.nb) * bpp_;
    if (need > p_.budget_bytes) {
      // the estimate grew past the budget after submission: never admitted
      results_.push_back(result_of(q, PRTCL_GPU_REQUEST_REJECTED, false));
      pending_.pop_front();
      continue;
    }
    if (held_ + need > p_.budget_bytes) break;
    // the request leaves the queue only once the batch holds it
    int64_t sid = b_->add(q.xf.data(), q.nf, q.xb.data(), q.nb);
    Request r = std::move(q);
    pending_.pop_front();
    r.sid = sid;
    r.admitted = t;
    std::vector<float>().swap(r.xf);
    std::vector<float>().swap(r.xb);
    running_.push_back(std::move(r));
    held_ = double(b_->device_bytes());
    size_t parts = 0;
    for (auto const &x : running_) parts += x.nf + x.nb;
    if (parts) bpp_ = std::max(bpp_, held_ / double(parts));
  }
  if (running_.empty()) return false;
  // 2. one step of every resident scene; if it fails, the resident scenes'
  // state is undefined: retire them all as failed, then report the error
  try {
    b_->step(1);
  } catch (std::exception const &) {
    for (auto &x : running_) {
      results_.push_back(result_of(x, PRTCL_GPU_REQUEST_FAILED, true));
      drop_scene(x.sid);
    }
    running_.clear();
    held_ = 0.0;
    throw;
  }
  steps_run_++;
  for (auto &x : running_) {
    particle_steps_ += int64_t(x.nf);
    x.done++;
  }
  // 3. retirements, in admission order; a request leaves the resident set
  // only once its result is stored and its scene removed
  bool retired = false;
  for (size_t k = 0; k < running_.size();) {
    Request &x = running_[k];
    if (x.done < x.steps) {
      ++k;
      continue;
    }
    // a failure to read the results fails this request alone: it is
    // retired all the same, so it is never stepped again
    bool ok = true;
    std::vector<float> xs;
    try {
      if (p_.keep_results) {
        xs.resize(3 * x.nf);
        b_->download_positions(x.sid, xs.data(), x.nf);
      } else {
        b_->synchronize();
      }
    } catch (std::exception const &) {
      ok = false;
      xs.clear();
    }
    Result res = result_of(x, ok ? PRTCL_GPU_REQUEST_DONE : PRTCL_GPU_REQUEST_FAILED, true);
    if (res.r.status == PRTCL_GPU_REQUEST_DONE) res.x = std::move(xs);
    drop_scene(x.sid);
    results_.push_back(std::move(res));
    running_.erase(running_.begin() + std::ptrdiff_t(k));
    retired = true;
  }
  if (retired) held_ = running_.empty() ? 0.0 : double(b_->device_bytes());
  return true;
}

prtcl_gpu_server_status Server::status() const {
  prtcl_gpu_server_status s{};
  s.pending = int64_t(pending_.size());
  s.running = int64_t(running_.size());
  s.results = int64_t(results_.size());
  s.steps_run = steps_run_;
  s.particle_steps = particle_steps_;
  s.held_bytes = int64_t(held_);
  s.next_arrival = pending_.empty() ? std::numeric_limits<double>::infinity() : pending_.front().arrival;
  return s;
}

bool Server::next_result(prtcl_gpu_request_result &out, float *x, size_t capacity) {
  if (results_.empty()) return false;
  Result &r = results_.front();
  if (x) {
    if (capacity < size_t(r.r.fluid)) throw Error("server: result buffer smaller than the request's fluid count");
    if (!r.x.empty()) std::copy(r.x.begin(), r.x.end(), x);
    else std::fill(x, x + 3 * size_t(r.r.fluid), 0.0f);
  }
  out = r.r;
  results_.pop_front();
  return true;
}

} // namespace prtcl_gpu
