// Serving: continuous batching of simulation requests over a batch of
// scenes (batch.hpp).  The reference runs one scene per process
// (share/scripts/prtcl-lua.example.lua:363-461); a server keeps every
// admitted request resident in one batch and steps all of them together,
// one step per turn, admitting arrived requests within a device-memory
// budget and retiring finished ones between turns.  The rules of a turn are
// those of the C ABI (include/prtcl_gpu.h, prtcl_gpu_server_*).
#pragma once

#include "../../include/prtcl_gpu.h"

#include <chrono>
#include <cstddef>
#include <deque>
#include <memory>
#include <vector>

namespace prtcl_gpu {

// What a server needs of a batch: the device batch, or one the caller
// supplies through callbacks (another backend, or a stand-in in host tests).
class ServeBatch {
public:
  virtual ~ServeBatch() = default;
  virtual int64_t add(float const *xf, size_t nf, float const *xb, size_t nb) = 0;
  virtual void remove(int64_t id) = 0;
  virtual void step(int k) = 0;
  virtual void synchronize() = 0;
  virtual size_t device_bytes() = 0;
  virtual prtcl_gpu_scene_info info(int64_t id) = 0;
  virtual void download_positions(int64_t id, float *host, size_t n) = 0;
};
std::unique_ptr<ServeBatch> device_serve_batch(prtcl_gpu_batch_params const &p);
std::unique_ptr<ServeBatch> callback_serve_batch(prtcl_gpu_server_batch_ops const &ops, void *user);

class Server {
public:
  Server(std::unique_ptr<ServeBatch> batch, prtcl_gpu_server_params const &p);
  void submit(int64_t rid, double arrival, float const *xf, size_t nf, float const *xb, size_t nb, int64_t steps);
  // one turn; false when nothing was resident to step
  bool turn();
  prtcl_gpu_server_status status() const;
  // retire a queued or resident request as cancelled; false if none has the id
  bool cancel(int64_t rid);
  // the oldest unread result, its positions copied to `x` when non-null
  bool next_result(prtcl_gpu_request_result &out, float *x, size_t capacity);

private:
  struct Request {
    int64_t rid = 0, steps = 0, done = 0, sid = 0;
    double arrival = 0.0, admitted = 0.0;
    size_t nf = 0, nb = 0;
    std::vector<float> xf, xb; // until admitted
  };
  struct Result {
    prtcl_gpu_request_result r{};
    std::vector<float> x;
  };
  double now() const;
  // a result for a request leaving the queue or the resident set
  Result result_of(Request const &x, int32_t status, bool resident);
  // remove a scene from the batch; on failure, retried at later turns
  void drop_scene(int64_t sid);

  std::unique_ptr<ServeBatch> b_;
  prtcl_gpu_server_params p_;
  std::chrono::steady_clock::time_point t0_;
  std::deque<Request> pending_;  // arrival order, ties in submission order
  std::vector<Request> running_; // admission order
  std::deque<Result> results_;
  std::vector<int64_t> orphans_; // scenes the batch failed to remove
  double held_ = 0.0, bpp_ = 0.0;
  int64_t steps_run_ = 0, particle_steps_ = 0;
};

} // namespace prtcl_gpu
