// Scheme runtime: the device counterpart of prtcl::SchemeBase and
// prtcl::SchemeRegistry (schemes/scheme_base.hpp:18-105).
//
// A scheme is created by its full name, e.g.
//   "prtcl::schemes::iisph[T=f32, N=3, K=Cubic Spline]"
// (schemes/iisph.hpp:519-525), Load()s a model (creating the fields it uses,
// as the generated Load does, schemes/iisph.hpp:134-185) and runs procedures
// by name.  Unknown names raise "procedure does not exist" /
// "scheme is not registered" like the reference.
#pragma once

#include "nhood.hpp"

#include <functional>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace prtcl_gpu {

class Scheme {
public:
  virtual ~Scheme() = default;
  virtual std::string name() const = 0;
  std::string full_name() const { return "prtcl::schemes::" + name() + "[T=f32, N=3, K=Cubic Spline]"; }
  virtual void load(Model &m) = 0;
  void run(std::string const &procedure, Nhood &nh, cudaStream_t s);
  std::vector<std::string> procedure_names() const;
  virtual std::string source() const = 0;
  Model *model() const { return model_; }

protected:
  using Proc = std::function<void(Nhood &, cudaStream_t)>;
  void reg(std::string const &n, Proc p) { procs_[n] = std::move(p); }
  void bind(Model &m) {
    model_ = &m;
    layout_version_ = m.layout_version;
  }
  Model *model_ = nullptr;
  uint64_t layout_version_ = 0;

private:
  std::map<std::string, Proc> procs_;
};

std::unique_ptr<Scheme> new_scheme(std::string const &full_name);
std::vector<std::string> scheme_names();

// Schemes added at run time: the generated plugins (schemes compiled from
// the scheme language) register a factory per scheme when they are loaded.
// A name already taken is an error.
using SchemeFactory = std::function<std::unique_ptr<Scheme>()>;
void register_scheme(std::string const &full_name, SchemeFactory f);

} // namespace prtcl_gpu
