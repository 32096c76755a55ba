// Batched scenes: many independent dam-break scenes resident on the device,
// stepped together by the procedures of the reference's step loop
// (share/scripts/prtcl-lua.example.lua:363-461).
//
// Layout.  One model holds every scene: group "b" (boundary) and group "f"
// (fluid, tag dynamic), each split into per-scene segments (slots), the
// ranges in slot order.  The neighbourhood puts the slot above the Z-order
// bits of the cell key, so a scene's cells, their order, their adjacency and
// every neighbour list are those of the scene run alone (indices shifted by
// the scene's range).  The per-particle procedures run as one launch over
// all scenes; the relaxed-Jacobi and PCG loops reduce and decide per slot.
// Permutes follow each scene's own step count.  Together this makes a
// scene's results independent of the other scenes and of when it was added.
//
// Composition changes (added and removed scenes) are applied lazily at the
// next step or query: fields are remapped into the new ranges, new scenes
// are uploaded and set up (update, permute of the new slots, boundary
// volumes) as the reference's set-up does (prtcl-lua.example.lua:196-316).
#pragma once

#include "../../include/prtcl_gpu.h"
#include "schemes.hpp"

#include <memory>
#include <string>
#include <vector>

namespace prtcl_gpu {

class Batch {
public:
  explicit Batch(prtcl_gpu_batch_params const &p);
  ~Batch();
  Batch(Batch const &) = delete;
  Batch &operator=(Batch const &) = delete;

  int64_t add(float const *xf, size_t nf, float const *xb, size_t nb);
  void remove(int64_t id);
  void step(int k);
  void synchronize();
  prtcl_gpu_scene_info info(int64_t id);
  void download(int64_t id, std::string const &field, void *host, size_t n);
  size_t scene_count() const;
  void particles(int64_t &nf, int64_t &nb);
  size_t device_bytes();
  Model &model() { return m_; }

private:
  struct Scene {
    int64_t id = 0;
    uint32_t slot = 0;
    size_t nf = 0, nb = 0;
    int64_t steps = 0;
    int since_permute = 0;
    bool fresh = true;            // not yet in the device layout
    std::vector<float> xf, xb;    // positions until uploaded
  };
  void commit();
  Scene &find(int64_t id);
  void run(Scheme &s, char const *proc);
  void set_global(char const *name, void const *value);

  prtcl_gpu_batch_params p_;
  Model m_;
  Nhood nh_;
  std::unique_ptr<Scheme> density_, gravity_, euler_, iisph_, wkbb18_, aiast12_;
  Group *f_ = nullptr, *b_ = nullptr;
  std::vector<Scene> scenes_;     // live and pending scenes, in slot order after commit()
  std::vector<int64_t> removed_;  // pending removals
  bool dirty_ = false;
  int64_t next_id_ = 1;
  uint32_t slots_ = 0;            // slot count of the device layout
  double t_ = 0.0;                // batch clock (double, like the script's clock)
  std::vector<uint32_t> fstart_, bstart_; // per slot ranges of the device layout
};

} // namespace prtcl_gpu
