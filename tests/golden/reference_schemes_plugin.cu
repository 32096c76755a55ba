// Generated by tests/golden/make_reference_schemes.py with prtcl_gb300.dsl from the
// reference's share/schemes/{aiast12, density, gravity, iisph, symplectic_euler, wkbb18}.prtcl (schemes renamed
// ref_<name>).  Test fixture: do not edit.
// Generated from the scheme language by prtcl_gb300.dsl.
#include "dsl_device.cuh"
#include "schemes.hpp"

#include <memory>

// scheme aiast12
namespace prtcl_gpu {
namespace gen_aiast12_137ff5928731 {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_boundary {
  uint32_t n;
  int index;
  float4 *v_x;
  float *v_V;
};
struct G_boundary_all {
  int count;
  G_boundary g[kMaxGroups];
};
struct Glob {
  SReal g_h;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_compute_volume_p0(G_boundary p, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_V, i, float(float(0)));
    for (int q2_ = 0; q2_ < nb_boundary.count; ++q2_) { // foreach boundary neighbor b_b
      G_boundary const &n = nb_boundary.g[q2_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t3_ = rd(p.v_V, i); add_to(t3_, kernel_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))); wr(p.v_V, i, t3_); }
      });
    }
    wr(p.v_V, i, float((float(1) / rd(p.v_V, i))));
  }
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("compute_volume", [this](Nhood &nh, cudaStream_t s) { proc_compute_volume(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_aiast12"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_h_ = &m.add_global("smoothing_scale", parse_field_type("f32", 0, nullptr));
    sel_boundary.clear();
    for (Group *grp : m.groups_by_index()) {
      if ((grp->type == "boundary")) {
        if (sel_boundary.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_boundary.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("volume", parse_field_type("f32", 0, nullptr));
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_h_ = nullptr;
  std::vector<Group *> sel_boundary;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_h = SReal{static_cast<float *>(model_->small_ptr(*glob_h_))};
    return r;
  }
  G_boundary mk_boundary(Group *grp) const {
    G_boundary r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_V = grp->varying.at("volume");
    r.v_V = static_cast<float *>(f_V.d);
    return r;
  }
  G_boundary_all all_boundary() const {
    G_boundary_all r{};
    r.count = int(sel_boundary.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_boundary(sel_boundary[k]);
    return r;
  }
  void proc_compute_volume(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach boundary particle b
      for (Group *pg : sel_boundary) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_compute_volume_p0<<<blocks_, kGenNT, 0, s>>>(mk_boundary(pg), all_boundary(), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_boundary) pg->varying.at("volume").version++;
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_aiast12_137ff5928731
} // namespace prtcl_gpu

// scheme density
namespace prtcl_gpu {
namespace gen_density_51043b23b2ed {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_fluid {
  uint32_t n;
  int index;
  float4 *v_x;
  float *v_rho;
  float *v_m;
  SReal u_rho0;
};
struct G_fluid_all {
  int count;
  G_fluid g[kMaxGroups];
};
struct G_boundary {
  uint32_t n;
  int index;
  float4 *v_x;
  float *v_V;
};
struct G_boundary_all {
  int count;
  G_boundary g[kMaxGroups];
};
struct Glob {
  SReal g_h;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_compute_density_p0(G_fluid p, G_fluid_all nb_fluid, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_rho, i, float(float(0)));
    for (int q2_ = 0; q2_ < nb_fluid.count; ++q2_) { // foreach fluid neighbor f_f
      G_fluid const &n = nb_fluid.g[q2_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t3_ = rd(p.v_rho, i); add_to(t3_, (rd(n.v_m, j) * kernel_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_rho, i, t3_); }
      });
    }
    for (int q4_ = 0; q4_ < nb_boundary.count; ++q4_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q4_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t5_ = rd(p.v_rho, i); add_to(t5_, ((rd(n.v_V, j) * rd(p.u_rho0)) * kernel_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_rho, i, t5_); }
      });
    }
  }
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("compute_density", [this](Nhood &nh, cudaStream_t s) { proc_compute_density(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_density"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_h_ = &m.add_global("smoothing_scale", parse_field_type("f32", 0, nullptr));
    sel_fluid.clear();
    sel_boundary.clear();
    for (Group *grp : m.groups_by_index()) {
      if ((grp->type == "fluid")) {
        if (sel_fluid.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_fluid.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("density", parse_field_type("f32", 0, nullptr));
        grp->add_varying("mass", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("rest_density", parse_field_type("f32", 0, nullptr));
      }
      if ((grp->type == "boundary")) {
        if (sel_boundary.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_boundary.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("volume", parse_field_type("f32", 0, nullptr));
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_h_ = nullptr;
  std::vector<Group *> sel_fluid;
  std::vector<Group *> sel_boundary;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_h = SReal{static_cast<float *>(model_->small_ptr(*glob_h_))};
    return r;
  }
  G_fluid mk_fluid(Group *grp) const {
    G_fluid r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_rho = grp->varying.at("density");
    r.v_rho = static_cast<float *>(f_rho.d);
    VaryingField &f_m = grp->varying.at("mass");
    r.v_m = static_cast<float *>(f_m.d);
    r.u_rho0 = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("rest_density")))};
    return r;
  }
  G_fluid_all all_fluid() const {
    G_fluid_all r{};
    r.count = int(sel_fluid.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_fluid(sel_fluid[k]);
    return r;
  }
  G_boundary mk_boundary(Group *grp) const {
    G_boundary r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_V = grp->varying.at("volume");
    r.v_V = static_cast<float *>(f_V.d);
    return r;
  }
  G_boundary_all all_boundary() const {
    G_boundary_all r{};
    r.count = int(sel_boundary.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_boundary(sel_boundary[k]);
    return r;
  }
  void proc_compute_density(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach fluid particle f
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_compute_density_p0<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_fluid(), all_boundary(), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_fluid) pg->varying.at("density").version++;
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_density_51043b23b2ed
} // namespace prtcl_gpu

// scheme gravity
namespace prtcl_gpu {
namespace gen_gravity_20408f2f18b0 {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_dynamic {
  uint32_t n;
  int index;
  float4 *v_x;
  float4 *v_a;
};
struct G_dynamic_all {
  int count;
  G_dynamic g[kMaxGroups];
};
struct Glob {
  SVec g_g;
  SVec g_c;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_initialize_acceleration_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_a, i, f3(rd(g.g_g)));
  }
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    { f3 t2_ = rd(p.v_a, i); add_to(t2_, rd(g.g_g)); wr(p.v_a, i, t2_); }
  }
}

__global__ void __launch_bounds__(kGenNT) k_initialize_axial_acceleration_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    f3 l_xc = (rd(p.v_x, i) - rd(g.g_c));
    f3 l_g_n = (rd(g.g_g) * reciprocal_or_zero(norm(rd(g.g_g)), float(1e-9)));
    f3 l_xc_o = (l_xc - (dot(l_xc, l_g_n) * l_g_n));
    wr(p.v_a, i, f3((((-norm(rd(g.g_g))) * l_xc_o) * reciprocal_or_zero(norm(l_xc_o), float(1e-9)))));
  }
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("initialize_acceleration", [this](Nhood &nh, cudaStream_t s) { proc_initialize_acceleration(nh, s); });
    reg("accumulate_acceleration", [this](Nhood &nh, cudaStream_t s) { proc_accumulate_acceleration(nh, s); });
    reg("initialize_axial_acceleration", [this](Nhood &nh, cudaStream_t s) { proc_initialize_axial_acceleration(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_gravity"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_g_ = &m.add_global("gravity", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
    glob_c_ = &m.add_global("gravity_center", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
    sel_dynamic.clear();
    for (Group *grp : m.groups_by_index()) {
      if (grp->has_tag("dynamic")) {
        if (sel_dynamic.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_dynamic.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("acceleration", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_g_ = nullptr;
  SmallField *glob_c_ = nullptr;
  std::vector<Group *> sel_dynamic;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_g = SVec{static_cast<float *>(model_->small_ptr(*glob_g_))};
    r.g_c = SVec{static_cast<float *>(model_->small_ptr(*glob_c_))};
    return r;
  }
  G_dynamic mk_dynamic(Group *grp) const {
    G_dynamic r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_a = grp->varying.at("acceleration");
    r.v_a = static_cast<float4 *>(f_a.d);
    return r;
  }
  G_dynamic_all all_dynamic() const {
    G_dynamic_all r{};
    r.count = int(sel_dynamic.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_dynamic(sel_dynamic[k]);
    return r;
  }
  void proc_initialize_acceleration(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle f
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_initialize_acceleration_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("acceleration").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_accumulate_acceleration(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle f
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_accumulate_acceleration_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("acceleration").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_initialize_axial_acceleration(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle f
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_initialize_axial_acceleration_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("acceleration").version++;
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_gravity_20408f2f18b0
} // namespace prtcl_gpu

// scheme iisph
namespace prtcl_gpu {
namespace gen_iisph_177f18681cf7 {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_fluid {
  uint32_t n;
  int index;
  float4 *v_x;
  float4 *v_v;
  float4 *v_a;
  float *v_rho;
  float *v_p;
  float *v_m;
  SReal u_rho0;
  float4 *v_c;
  float *v_s;
  float *v_AA;
  float *v_Ap;
};
struct G_fluid_all {
  int count;
  G_fluid g[kMaxGroups];
};
struct G_boundary {
  uint32_t n;
  int index;
  float4 *v_x;
  float *v_V;
};
struct G_boundary_all {
  int count;
  G_boundary g[kMaxGroups];
};
struct Glob {
  SVec g_g;
  SReal g_h;
  SReal g_dt;
  SReal g_omega;
  SReal g_aprde;
  SInt g_nprde;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_setup_p0(G_fluid p, G_fluid_all nb_fluid, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_c, i, f3(zeros<f3>()));
    for (int q2_ = 0; q2_ < nb_fluid.count; ++q2_) { // foreach fluid neighbor f_f
      G_fluid const &n = nb_fluid.g[q2_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t3_ = rd(p.v_c, i); sub_from(t3_, ((rd(n.v_m, j) / (rd(p.v_rho, i) * rd(p.v_rho, i))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_c, i, t3_); }
      });
    }
    for (int q4_ = 0; q4_ < nb_boundary.count; ++q4_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q4_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t5_ = rd(p.v_c, i); sub_from(t5_, ((((float(0.7) * float(2)) * rd(p.u_rho0)) * (rd(n.v_V, j) / (rd(p.v_rho, i) * rd(p.v_rho, i)))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_c, i, t5_); }
      });
    }
  }
}

__global__ void k_setup_s1(Glob g, float *fr) {
  wr(g.g_nprde, int(zeros<int>()));
}

__global__ void __launch_bounds__(kGenNT) k_setup_p2(G_fluid p, G_fluid_all nb_fluid, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  double r0_ = 0.0;
  if (i < p.n) {
    wr(p.v_p, i, float(float(0)));
    wr(p.v_s, i, float(float(0)));
    wr(p.v_AA, i, float(float(0)));
    for (int q10_ = 0; q10_ < nb_fluid.count; ++q10_) { // foreach fluid neighbor f_f
      G_fluid const &n = nb_fluid.g[q10_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t11_ = rd(p.v_s, i); add_to(t11_, (rd(n.v_m, j) * dot((rd(p.v_v, i) - rd(n.v_v, j)), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_s, i, t11_); }
        { float t12_ = rd(p.v_AA, i); add_to(t12_, (rd(n.v_m, j) * dot(rd(p.v_c, i), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_AA, i, t12_); }
        { float t13_ = rd(p.v_AA, i); sub_from(t13_, ((rd(n.v_m, j) * (rd(p.v_m, i) / (rd(p.v_rho, i) * rd(p.v_rho, i)))) * norm_squared(kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_AA, i, t13_); }
      });
    }
    for (int q14_ = 0; q14_ < nb_boundary.count; ++q14_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q14_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t15_ = rd(p.v_s, i); add_to(t15_, ((rd(p.u_rho0) * rd(n.v_V, j)) * dot((rd(p.v_v, i) - zeros<f3>()), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_s, i, t15_); }
        { float t16_ = rd(p.v_AA, i); add_to(t16_, ((rd(p.u_rho0) * rd(n.v_V, j)) * dot(rd(p.v_c, i), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_AA, i, t16_); }
      });
    }
    wr(p.v_s, i, float(((rd(p.u_rho0) - rd(p.v_rho, i)) - ((rd(g.g_dt) * (rd(p.u_rho0) / rd(p.v_rho, i))) * rd(p.v_s, i)))));
    { float t18_ = rd(p.v_AA, i); mul_by(t18_, ((rd(g.g_dt) * rd(g.g_dt)) * (rd(p.u_rho0) / rd(p.v_rho, i)))); wr(p.v_AA, i, t18_); }
    r0_ += double(ones<int>());
  }
  __shared__ double sh_[32];
  { double b_ = block_sum(r0_, sh_); if (threadIdx.x == 0) red[size_t(0) * red_cap + red_off + blockIdx.x] = b_; }
}

__global__ void k_setup_p2_f(Glob g, float *fr, double const *red, uint32_t red_cap, uint32_t nparts) {
  { // reduce +=
    double const *pr_ = red + size_t(0) * red_cap;
    double a_ = 0.0;
    for (uint32_t b = 0; b < nparts; ++b) a_ += pr_[b];
    double v_ = double(rd(g.g_nprde)) + a_;
    wr(g.g_nprde, int(llrint(v_)));
  }
}

__global__ void __launch_bounds__(kGenNT) k_iteration_pressure_acceleration_p0(G_fluid p, G_fluid_all nb_fluid, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_a, i, f3(zeros<f3>()));
    for (int q20_ = 0; q20_ < nb_fluid.count; ++q20_) { // foreach fluid neighbor f_f
      G_fluid const &n = nb_fluid.g[q20_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t21_ = rd(p.v_a, i); sub_from(t21_, ((rd(n.v_m, j) * ((rd(p.v_p, i) / (rd(p.v_rho, i) * rd(p.v_rho, i))) + (rd(n.v_p, j) / (rd(n.v_rho, j) * rd(n.v_rho, j))))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_a, i, t21_); }
      });
    }
    for (int q22_ = 0; q22_ < nb_boundary.count; ++q22_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q22_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t23_ = rd(p.v_a, i); sub_from(t23_, ((((float(0.7) * rd(p.u_rho0)) * rd(n.v_V, j)) * ((float(2) * rd(p.v_p, i)) / (rd(p.v_rho, i) * rd(p.v_rho, i)))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); wr(p.v_a, i, t23_); }
      });
    }
  }
}

__global__ void __launch_bounds__(kGenNT) k_iteration_pressure_p0(G_fluid p, G_fluid_all nb_fluid, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  double r0_ = 0.0;
  if (i < p.n) {
    wr(p.v_Ap, i, float(float(0)));
    for (int q25_ = 0; q25_ < nb_fluid.count; ++q25_) { // foreach fluid neighbor f_f
      G_fluid const &n = nb_fluid.g[q25_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t26_ = rd(p.v_Ap, i); add_to(t26_, (rd(n.v_m, j) * dot((rd(p.v_a, i) - rd(n.v_a, j)), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_Ap, i, t26_); }
      });
    }
    for (int q27_ = 0; q27_ < nb_boundary.count; ++q27_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q27_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { float t28_ = rd(p.v_Ap, i); add_to(t28_, ((rd(p.u_rho0) * rd(n.v_V, j)) * dot((rd(p.v_a, i) - zeros<f3>()), kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h))))); wr(p.v_Ap, i, t28_); }
      });
    }
    { float t29_ = rd(p.v_Ap, i); mul_by(t29_, ((rd(g.g_dt) * rd(g.g_dt)) * (rd(p.u_rho0) / rd(p.v_rho, i)))); wr(p.v_Ap, i, t29_); }
    wr(p.v_p, i, float((max<float>(float(0), (rd(p.v_p, i) + ((rd(g.g_omega) * (rd(p.v_s, i) - rd(p.v_Ap, i))) * reciprocal_or_zero(rd(p.v_AA, i), float(1e-9))))) * unit_step_l(float(float(1e-9)), float(cabs(rd(p.v_AA, i)))))));
    r0_ += double((((rd(p.v_Ap, i) - rd(p.v_s, i)) / rd(p.u_rho0)) * unit_step_l(float(float(1e-9)), float(rd(p.v_p, i)))));
  }
  __shared__ double sh_[32];
  { double b_ = block_sum(r0_, sh_); if (threadIdx.x == 0) red[size_t(0) * red_cap + red_off + blockIdx.x] = b_; }
}

__global__ void k_iteration_pressure_p0_f(Glob g, float *fr, double const *red, uint32_t red_cap, uint32_t nparts) {
  { // reduce +=
    double const *pr_ = red + size_t(0) * red_cap;
    double a_ = 0.0;
    for (uint32_t b = 0; b < nparts; ++b) a_ += pr_[b];
    double v_ = double(rd(g.g_aprde)) + a_;
    wr(g.g_aprde, float(v_));
  }
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("setup", [this](Nhood &nh, cudaStream_t s) { proc_setup(nh, s); });
    reg("iteration_pressure_acceleration", [this](Nhood &nh, cudaStream_t s) { proc_iteration_pressure_acceleration(nh, s); });
    reg("iteration_pressure", [this](Nhood &nh, cudaStream_t s) { proc_iteration_pressure(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_iisph"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_g_ = &m.add_global("gravity", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
    glob_h_ = &m.add_global("smoothing_scale", parse_field_type("f32", 0, nullptr));
    glob_dt_ = &m.add_global("time_step", parse_field_type("f32", 0, nullptr));
    glob_omega_ = &m.add_global("iisph_relaxation", parse_field_type("f32", 0, nullptr));
    glob_aprde_ = &m.add_global("iisph_aprde", parse_field_type("f32", 0, nullptr));
    glob_nprde_ = &m.add_global("iisph_nprde", parse_field_type("i32", 0, nullptr));
    sel_fluid.clear();
    sel_boundary.clear();
    for (Group *grp : m.groups_by_index()) {
      if ((grp->type == "fluid")) {
        if (sel_fluid.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_fluid.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("velocity", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("acceleration", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("density", parse_field_type("f32", 0, nullptr));
        grp->add_varying("pressure", parse_field_type("f32", 0, nullptr));
        grp->add_varying("mass", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("rest_density", parse_field_type("f32", 0, nullptr));
        grp->add_varying("iisph_helper_c", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("iisph_source_term", parse_field_type("f32", 0, nullptr));
        grp->add_varying("iisph_diagonal_element", parse_field_type("f32", 0, nullptr));
        grp->add_varying("iisph_right_hand_side", parse_field_type("f32", 0, nullptr));
      }
      if ((grp->type == "boundary")) {
        if (sel_boundary.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_boundary.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("volume", parse_field_type("f32", 0, nullptr));
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_g_ = nullptr;
  SmallField *glob_h_ = nullptr;
  SmallField *glob_dt_ = nullptr;
  SmallField *glob_omega_ = nullptr;
  SmallField *glob_aprde_ = nullptr;
  SmallField *glob_nprde_ = nullptr;
  std::vector<Group *> sel_fluid;
  std::vector<Group *> sel_boundary;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_g = SVec{static_cast<float *>(model_->small_ptr(*glob_g_))};
    r.g_h = SReal{static_cast<float *>(model_->small_ptr(*glob_h_))};
    r.g_dt = SReal{static_cast<float *>(model_->small_ptr(*glob_dt_))};
    r.g_omega = SReal{static_cast<float *>(model_->small_ptr(*glob_omega_))};
    r.g_aprde = SReal{static_cast<float *>(model_->small_ptr(*glob_aprde_))};
    r.g_nprde = SInt{static_cast<int *>(model_->small_ptr(*glob_nprde_))};
    return r;
  }
  G_fluid mk_fluid(Group *grp) const {
    G_fluid r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_v = grp->varying.at("velocity");
    r.v_v = static_cast<float4 *>(f_v.d);
    VaryingField &f_a = grp->varying.at("acceleration");
    r.v_a = static_cast<float4 *>(f_a.d);
    VaryingField &f_rho = grp->varying.at("density");
    r.v_rho = static_cast<float *>(f_rho.d);
    VaryingField &f_p = grp->varying.at("pressure");
    r.v_p = static_cast<float *>(f_p.d);
    VaryingField &f_m = grp->varying.at("mass");
    r.v_m = static_cast<float *>(f_m.d);
    r.u_rho0 = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("rest_density")))};
    VaryingField &f_c = grp->varying.at("iisph_helper_c");
    r.v_c = static_cast<float4 *>(f_c.d);
    VaryingField &f_s = grp->varying.at("iisph_source_term");
    r.v_s = static_cast<float *>(f_s.d);
    VaryingField &f_AA = grp->varying.at("iisph_diagonal_element");
    r.v_AA = static_cast<float *>(f_AA.d);
    VaryingField &f_Ap = grp->varying.at("iisph_right_hand_side");
    r.v_Ap = static_cast<float *>(f_Ap.d);
    return r;
  }
  G_fluid_all all_fluid() const {
    G_fluid_all r{};
    r.count = int(sel_fluid.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_fluid(sel_fluid[k]);
    return r;
  }
  G_boundary mk_boundary(Group *grp) const {
    G_boundary r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_V = grp->varying.at("volume");
    r.v_V = static_cast<float *>(f_V.d);
    return r;
  }
  G_boundary_all all_boundary() const {
    G_boundary_all r{};
    r.count = int(sel_boundary.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_boundary(sel_boundary[k]);
    return r;
  }
  void proc_setup(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach fluid particle f
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_setup_p0<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_fluid(), all_boundary(), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_fluid) pg->varying.at("iisph_helper_c").version++;
    }
    k_setup_s1<<<1, 1, 0, s>>>(glob(), frame_);
    count_launch();
    { // foreach fluid particle f
      uint32_t off_ = 0, total_ = 0;
      for (Group *pg : sel_fluid) total_ += uint32_t((pg->count + kGenNT - 1) / kGenNT);
      ensure_red(1, total_);
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_setup_p2<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_fluid(), all_boundary(), glob(), lv_, frame_, red_, red_cap_, off_);
        count_launch();
        off_ += blocks_;
      }
      for (Group *pg : sel_fluid) pg->varying.at("pressure").version++;
      for (Group *pg : sel_fluid) pg->varying.at("iisph_source_term").version++;
      for (Group *pg : sel_fluid) pg->varying.at("iisph_diagonal_element").version++;
      k_setup_p2_f<<<1, 1, 0, s>>>(glob(), frame_, red_, red_cap_, total_);
      count_launch();
    }
    PG_LAUNCH_CHECK();
  }
  void proc_iteration_pressure_acceleration(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach fluid particle f
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_iteration_pressure_acceleration_p0<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_fluid(), all_boundary(), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_fluid) pg->varying.at("acceleration").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_iteration_pressure(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach fluid particle f
      uint32_t off_ = 0, total_ = 0;
      for (Group *pg : sel_fluid) total_ += uint32_t((pg->count + kGenNT - 1) / kGenNT);
      ensure_red(1, total_);
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_iteration_pressure_p0<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_fluid(), all_boundary(), glob(), lv_, frame_, red_, red_cap_, off_);
        count_launch();
        off_ += blocks_;
      }
      for (Group *pg : sel_fluid) pg->varying.at("iisph_right_hand_side").version++;
      for (Group *pg : sel_fluid) pg->varying.at("pressure").version++;
      k_iteration_pressure_p0_f<<<1, 1, 0, s>>>(glob(), frame_, red_, red_cap_, total_);
      count_launch();
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_iisph_177f18681cf7
} // namespace prtcl_gpu

// scheme symplectic_euler
namespace prtcl_gpu {
namespace gen_symplectic_euler_13eb52a9f28b {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_dynamic {
  uint32_t n;
  int index;
  float4 *v_x;
  float4 *v_v;
  float4 *v_a;
  float *v_t_birth;
};
struct G_dynamic_all {
  int count;
  G_dynamic g[kMaxGroups];
};
struct Glob {
  SReal g_dt;
  SReal g_t;
  SReal g_dt_fade;
  SReal g_max_speed;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_integrate_velocity_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    { f3 t1_ = rd(p.v_v, i); add_to(t1_, (rd(g.g_dt) * rd(p.v_a, i))); wr(p.v_v, i, t1_); }
  }
}

__global__ void __launch_bounds__(kGenNT) k_integrate_velocity_with_hard_fade_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    { f3 t2_ = rd(p.v_v, i); add_to(t2_, ((rd(g.g_dt) * rd(p.v_a, i)) * unit_step_l(float(float(0)), float(((rd(g.g_t) - rd(p.v_t_birth, i)) - rd(g.g_dt_fade)))))); wr(p.v_v, i, t2_); }
  }
}

__global__ void __launch_bounds__(kGenNT) k_integrate_velocity_with_smooth_fade_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    { f3 t3_ = rd(p.v_v, i); add_to(t3_, ((rd(g.g_dt) * rd(p.v_a, i)) * smoothstep((((rd(g.g_t) - rd(p.v_t_birth, i)) - rd(g.g_dt_fade)) / rd(g.g_dt_fade))))); wr(p.v_v, i, t3_); }
  }
}

__global__ void __launch_bounds__(kGenNT) k_integrate_position_p0(G_dynamic p, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  double r0_ = -INFINITY;
  if (i < p.n) {
    { f3 t4_ = rd(p.v_x, i); add_to(t4_, (rd(g.g_dt) * rd(p.v_v, i))); wr(p.v_x, i, t4_); }
    { double v_ = double(norm(rd(p.v_v, i))); r0_ = (r0_ < v_) ? v_ : r0_; }
  }
  __shared__ double sh_[32];
  { double b_ = block_reduce_max(r0_, sh_); if (threadIdx.x == 0) red[size_t(0) * red_cap + red_off + blockIdx.x] = b_; }
}

__global__ void k_integrate_position_p0_f(Glob g, float *fr, double const *red, uint32_t red_cap, uint32_t nparts) {
  { // reduce max=
    double const *pr_ = red + size_t(0) * red_cap;
    double v_ = double(rd(g.g_max_speed));
    for (uint32_t b = 0; b < nparts; ++b) if (v_ < pr_[b]) v_ = pr_[b];
    wr(g.g_max_speed, float(v_));
  }
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("integrate_velocity", [this](Nhood &nh, cudaStream_t s) { proc_integrate_velocity(nh, s); });
    reg("integrate_velocity_with_hard_fade", [this](Nhood &nh, cudaStream_t s) { proc_integrate_velocity_with_hard_fade(nh, s); });
    reg("integrate_velocity_with_smooth_fade", [this](Nhood &nh, cudaStream_t s) { proc_integrate_velocity_with_smooth_fade(nh, s); });
    reg("integrate_position", [this](Nhood &nh, cudaStream_t s) { proc_integrate_position(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_symplectic_euler"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_dt_ = &m.add_global("time_step", parse_field_type("f32", 0, nullptr));
    glob_t_ = &m.add_global("current_time", parse_field_type("f32", 0, nullptr));
    glob_dt_fade_ = &m.add_global("fade_duration", parse_field_type("f32", 0, nullptr));
    glob_max_speed_ = &m.add_global("maximum_speed", parse_field_type("f32", 0, nullptr));
    sel_dynamic.clear();
    for (Group *grp : m.groups_by_index()) {
      if (grp->has_tag("dynamic")) {
        if (sel_dynamic.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_dynamic.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("velocity", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("acceleration", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("time_of_birth", parse_field_type("f32", 0, nullptr));
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_dt_ = nullptr;
  SmallField *glob_t_ = nullptr;
  SmallField *glob_dt_fade_ = nullptr;
  SmallField *glob_max_speed_ = nullptr;
  std::vector<Group *> sel_dynamic;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_dt = SReal{static_cast<float *>(model_->small_ptr(*glob_dt_))};
    r.g_t = SReal{static_cast<float *>(model_->small_ptr(*glob_t_))};
    r.g_dt_fade = SReal{static_cast<float *>(model_->small_ptr(*glob_dt_fade_))};
    r.g_max_speed = SReal{static_cast<float *>(model_->small_ptr(*glob_max_speed_))};
    return r;
  }
  G_dynamic mk_dynamic(Group *grp) const {
    G_dynamic r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_v = grp->varying.at("velocity");
    r.v_v = static_cast<float4 *>(f_v.d);
    VaryingField &f_a = grp->varying.at("acceleration");
    r.v_a = static_cast<float4 *>(f_a.d);
    VaryingField &f_t_birth = grp->varying.at("time_of_birth");
    r.v_t_birth = static_cast<float *>(f_t_birth.d);
    return r;
  }
  G_dynamic_all all_dynamic() const {
    G_dynamic_all r{};
    r.count = int(sel_dynamic.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_dynamic(sel_dynamic[k]);
    return r;
  }
  void proc_integrate_velocity(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle i
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_integrate_velocity_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("velocity").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_integrate_velocity_with_hard_fade(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle i
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_integrate_velocity_with_hard_fade_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("velocity").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_integrate_velocity_with_smooth_fade(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle i
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_integrate_velocity_with_smooth_fade_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_dynamic) pg->varying.at("velocity").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_integrate_position(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach dynamic particle i
      uint32_t off_ = 0, total_ = 0;
      for (Group *pg : sel_dynamic) total_ += uint32_t((pg->count + kGenNT - 1) / kGenNT);
      ensure_red(1, total_);
      for (Group *pg : sel_dynamic) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView lv_{};
        k_integrate_position_p0<<<blocks_, kGenNT, 0, s>>>(mk_dynamic(pg), glob(), lv_, frame_, red_, red_cap_, off_);
        count_launch();
        off_ += blocks_;
      }
      for (Group *pg : sel_dynamic) pg->varying.at("position").version++;
      k_integrate_position_p0_f<<<1, 1, 0, s>>>(glob(), frame_, red_, red_cap_, total_);
      count_launch();
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_symplectic_euler_13eb52a9f28b
} // namespace prtcl_gpu

// scheme wkbb18
namespace prtcl_gpu {
namespace gen_wkbb18_1c18b6a3b4c9 {
using namespace ::prtcl_gpu::dsl;
constexpr int kGenNT = 128;

struct G_fluid {
  uint32_t n;
  int index;
  float4 *v_x;
  float4 *v_v;
  float4 *v_a;
  float *v_rho;
  float *v_m;
  SReal u_rho0;
  SReal u_mu;
  float4 *v_vd;
  Planar9 v_sp;
  float *v_t_birth;
  SReal u_pcg_max_error;
  SInt u_pcg_max_iters;
  SInt u_pcg_iterations;
};
struct G_fluid_all {
  int count;
  G_fluid g[kMaxGroups];
};
struct G_boundary {
  uint32_t n;
  int index;
  float4 *v_x;
  float *v_V;
  SReal u_mu;
};
struct G_boundary_all {
  int count;
  G_boundary g[kMaxGroups];
};
struct Glob {
  SReal g_h;
  SReal g_dt;
  SReal g_t;
  SReal g_dt_fade;
  int unused_;
};

__global__ void __launch_bounds__(kGenNT) k_compute_diagonal_p0(G_fluid p, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, double *red, uint32_t red_cap, uint32_t red_off) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i < p.n) {
    wr(p.v_sp, i, M3(zeros<M3>()));
    { // foreach _ neighbor f_f
      G_fluid const &n = p;
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { M3 t2_ = rd(p.v_sp, i); add_to(t2_, ((((float(10) * (rd(p.u_mu) / rd(p.v_rho, i))) * (rd(n.v_m, j) / rd(n.v_rho, j))) / (norm_squared((rd(p.v_x, i) - rd(n.v_x, j))) + ((float(0.01) * rd(g.g_h)) * rd(g.g_h)))) * outer_product(kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)), (rd(p.v_x, i) - rd(n.v_x, j))))); wr(p.v_sp, i, t2_); }
      });
    }
    for (int q3_ = 0; q3_ < nb_boundary.count; ++q3_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q3_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { M3 t4_ = rd(p.v_sp, i); add_to(t4_, ((((float(10) * (rd(n.u_mu) / rd(p.v_rho, i))) * ((rd(p.u_rho0) * rd(n.v_V, j)) / rd(p.v_rho, i))) / (norm_squared((rd(p.v_x, i) - rd(n.v_x, j))) + ((float(0.01) * rd(g.g_h)) * rd(g.g_h)))) * outer_product(kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)), (rd(p.v_x, i) - rd(n.v_x, j))))); wr(p.v_sp, i, t4_); }
      });
    }
    wr(p.v_sp, i, M3(invert((identity3() - (rd(g.g_dt) * rd(p.v_sp, i))))));
  }
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_v0_right_hand_side(G_fluid p, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, float4 *into_, float4 const *with_) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i >= p.n) return;
  (void)into_;
  (void)with_;
    f3 l_a_b = zeros<f3>();
    f3 l_v_f_b = zeros<f3>();
    for (int q6_ = 0; q6_ < nb_boundary.count; ++q6_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q6_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t7_ = l_a_b; add_to(t7_, (((((float(10) * (rd(n.u_mu) / rd(p.v_rho, i))) * ((rd(p.u_rho0) * rd(n.v_V, j)) / rd(p.v_rho, i))) * dot(l_v_f_b, (rd(p.v_x, i) - rd(n.v_x, j)))) / (norm_squared((rd(p.v_x, i) - rd(n.v_x, j))) + ((float(0.01) * rd(g.g_h)) * rd(g.g_h)))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); l_a_b = t7_; }
      });
    }
    vst(into_, i, f3((rd(p.v_v, i) - (rd(g.g_dt) * l_a_b))));
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_v0_guess(G_fluid p, Glob g, NbrView L, float *fr, float4 *into_, float4 const *with_) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i >= p.n) return;
  (void)into_;
  (void)with_;
    vst(into_, i, f3(rd(p.v_v, i)));
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_v0_preconditioner(G_fluid p, Glob g, NbrView L, float *fr, float4 *into_, float4 const *with_) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i >= p.n) return;
  (void)into_;
  (void)with_;
    vst(into_, i, f3((rd(p.v_sp, i) * vld(with_, i))));
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_v0_system(G_fluid p, G_boundary_all nb_boundary, Glob g, NbrView L, float *fr, float4 *into_, float4 const *with_) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i >= p.n) return;
  (void)into_;
  (void)with_;
    f3 l_a_f = zeros<f3>();
    { // foreach _ neighbor f_f
      G_fluid const &n = p;
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t11_ = l_a_f; add_to(t11_, (((((float(10) * (rd(p.u_mu) / rd(p.v_rho, i))) * (rd(n.v_m, j) / rd(n.v_rho, j))) * dot((vld(with_, i) - vld(with_, j)), (rd(p.v_x, i) - rd(n.v_x, j)))) / (norm_squared((rd(p.v_x, i) - rd(n.v_x, j))) + ((float(0.01) * rd(g.g_h)) * rd(g.g_h)))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); l_a_f = t11_; }
      });
    }
    for (int q12_ = 0; q12_ < nb_boundary.count; ++q12_) { // foreach boundary neighbor f_b
      G_boundary const &n = nb_boundary.g[q12_];
      NbrList nl_ = nbr_list(L, n.index);
      if (nl_.cb) for_each_nbr(nl_, i, false, [&](uint32_t j, float) {
        { f3 t13_ = l_a_f; add_to(t13_, (((((float(10) * (rd(n.u_mu) / rd(p.v_rho, i))) * ((rd(p.u_rho0) * rd(n.v_V, j)) / rd(p.v_rho, i))) * dot(vld(with_, i), (rd(p.v_x, i) - rd(n.v_x, j)))) / (norm_squared((rd(p.v_x, i) - rd(n.v_x, j))) + ((float(0.01) * rd(g.g_h)) * rd(g.g_h)))) * kernel_gradient_h((rd(p.v_x, i) - rd(n.v_x, j)), rd(g.g_h)))); l_a_f = t13_; }
      });
    }
    vst(into_, i, f3((vld(with_, i) - (rd(g.g_dt) * l_a_f))));
}

__global__ void __launch_bounds__(kGenNT) k_accumulate_acceleration_v0_apply(G_fluid p, Glob g, NbrView L, float *fr, float4 *into_, float4 const *with_) {
  uint32_t i = blockIdx.x * kGenNT + threadIdx.x;
  if (i >= p.n) return;
  (void)into_;
  (void)with_;
    wr(p.v_vd, i, f3(((vld(with_, i) - rd(p.v_v, i)) * unit_step_l(float(float(0)), float(((rd(g.g_t) - rd(p.v_t_birth, i)) - rd(g.g_dt_fade)))))));
    wr(p.v_a, i, f3((rd(p.v_vd, i) / rd(g.g_dt))));
}

class Scheme_ : public Scheme {
public:
  Scheme_() {
    reg("compute_diagonal", [this](Nhood &nh, cudaStream_t s) { proc_compute_diagonal(nh, s); });
    reg("accumulate_acceleration", [this](Nhood &nh, cudaStream_t s) { proc_accumulate_acceleration(nh, s); });
  }
  ~Scheme_() override {
    if (frame_) cudaFree(frame_);
    if (red_) cudaFree(red_);
    if (pcg_buf_) cudaFree(pcg_buf_);
    if (pcg_part_) cudaFree(pcg_part_);
    if (pcg_state_) cudaFree(pcg_state_);
    if (pcg_stop_h_) cudaFreeHost(pcg_stop_h_);
  }
  std::string name() const override { return "ref_wkbb18"; }
  std::string source() const override { return R"prtcl_source((scheme source text not embedded in this build))prtcl_source"; }
  void load(Model &m) override {
    glob_h_ = &m.add_global("smoothing_scale", parse_field_type("f32", 0, nullptr));
    glob_dt_ = &m.add_global("time_step", parse_field_type("f32", 0, nullptr));
    glob_t_ = &m.add_global("current_time", parse_field_type("f32", 0, nullptr));
    glob_dt_fade_ = &m.add_global("fade_duration", parse_field_type("f32", 0, nullptr));
    sel_fluid.clear();
    sel_boundary.clear();
    for (Group *grp : m.groups_by_index()) {
      if ((grp->type == "fluid")) {
        if (sel_fluid.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_fluid.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("velocity", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("acceleration", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("density", parse_field_type("f32", 0, nullptr));
        grp->add_varying("mass", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("rest_density", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("dynamic_viscosity", parse_field_type("f32", 0, nullptr));
        grp->add_varying("wkbb18_velocity_delta", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("wkbb18_system_diagonal", [] { static int const e[] = {3, 3}; return parse_field_type("f32", 2, e); }());
        grp->add_varying("time_of_birth", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("wkbb18_maximum_error", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("wkbb18_maximum_iterations", parse_field_type("i32", 0, nullptr));
        grp->add_uniform("wkbb18_iterations", parse_field_type("i32", 0, nullptr));
      }
      if ((grp->type == "boundary")) {
        if (sel_boundary.size() == size_t(kMaxGroups)) throw Error("too many groups selected");
        sel_boundary.push_back(grp);
        grp->add_varying("position", [] { static int const e[] = {3}; return parse_field_type("f32", 1, e); }());
        grp->add_varying("volume", parse_field_type("f32", 0, nullptr));
        grp->add_uniform("dynamic_viscosity", parse_field_type("f32", 0, nullptr));
      }
    }
    if (!frame_) PG_CUDA(cudaMalloc(&frame_, 1 * 16 * sizeof(float)));
    bind(m);
  }
  std::string source_text() const { return source(); }

private:
  SmallField *glob_h_ = nullptr;
  SmallField *glob_dt_ = nullptr;
  SmallField *glob_t_ = nullptr;
  SmallField *glob_dt_fade_ = nullptr;
  std::vector<Group *> sel_fluid;
  std::vector<Group *> sel_boundary;
  float *frame_ = nullptr;
  double *red_ = nullptr;
  uint32_t red_cap_ = 0;
  void ensure_red(int nred, uint32_t parts) {
    if (parts <= red_cap_ && red_) return;
    if (red_) PG_CUDA(cudaFree(red_));
    red_cap_ = parts + parts / 4 + 64;
    PG_CUDA(cudaMalloc(&red_, size_t(1) * red_cap_ * sizeof(double)));
    (void)nred;
  }
  void *pcg_buf_ = nullptr;
  size_t pcg_vec_bytes_ = 0;
  double *pcg_part_ = nullptr;
  uint32_t pcg_part_cap_ = 0;
  PcgState *pcg_state_ = nullptr;
  int *pcg_stop_h_ = nullptr;
  // six solver vectors of `bytes` each, three partial-sum arrays of `parts` blocks
  void ensure_pcg(size_t bytes, uint32_t parts) {
    bytes = (bytes + 255) / 256 * 256;
    if (bytes > pcg_vec_bytes_) {
      if (pcg_buf_) PG_CUDA(cudaFree(pcg_buf_));
      pcg_vec_bytes_ = bytes + bytes / 4;
      PG_CUDA(cudaMalloc(&pcg_buf_, 6 * pcg_vec_bytes_));
    }
    if (parts > pcg_part_cap_) {
      if (pcg_part_) PG_CUDA(cudaFree(pcg_part_));
      pcg_part_cap_ = parts + parts / 4 + 64;
      PG_CUDA(cudaMalloc(&pcg_part_, 3 * size_t(pcg_part_cap_) * sizeof(double)));
    }
    if (!pcg_state_) PG_CUDA(cudaMalloc(&pcg_state_, sizeof(PcgState)));
    if (!pcg_stop_h_) PG_CUDA(cudaMallocHost(&pcg_stop_h_, sizeof(int)));
  }
  template <class S> S *pcg_vec(int k, uint32_t) const {
    return reinterpret_cast<S *>(static_cast<char *>(pcg_buf_) + size_t(k) * pcg_vec_bytes_);
  }
  Glob glob() const {
    Glob r{};
    r.g_h = SReal{static_cast<float *>(model_->small_ptr(*glob_h_))};
    r.g_dt = SReal{static_cast<float *>(model_->small_ptr(*glob_dt_))};
    r.g_t = SReal{static_cast<float *>(model_->small_ptr(*glob_t_))};
    r.g_dt_fade = SReal{static_cast<float *>(model_->small_ptr(*glob_dt_fade_))};
    return r;
  }
  G_fluid mk_fluid(Group *grp) const {
    G_fluid r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_v = grp->varying.at("velocity");
    r.v_v = static_cast<float4 *>(f_v.d);
    VaryingField &f_a = grp->varying.at("acceleration");
    r.v_a = static_cast<float4 *>(f_a.d);
    VaryingField &f_rho = grp->varying.at("density");
    r.v_rho = static_cast<float *>(f_rho.d);
    VaryingField &f_m = grp->varying.at("mass");
    r.v_m = static_cast<float *>(f_m.d);
    r.u_rho0 = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("rest_density")))};
    r.u_mu = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("dynamic_viscosity")))};
    VaryingField &f_vd = grp->varying.at("wkbb18_velocity_delta");
    r.v_vd = static_cast<float4 *>(f_vd.d);
    VaryingField &f_sp = grp->varying.at("wkbb18_system_diagonal");
    r.v_sp = Planar9{static_cast<float *>(f_sp.d), uint32_t(f_sp.cap)};
    VaryingField &f_t_birth = grp->varying.at("time_of_birth");
    r.v_t_birth = static_cast<float *>(f_t_birth.d);
    r.u_pcg_max_error = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("wkbb18_maximum_error")))};
    r.u_pcg_max_iters = SInt{static_cast<int *>(model_->small_ptr(grp->uniform.at("wkbb18_maximum_iterations")))};
    r.u_pcg_iterations = SInt{static_cast<int *>(model_->small_ptr(grp->uniform.at("wkbb18_iterations")))};
    return r;
  }
  G_fluid_all all_fluid() const {
    G_fluid_all r{};
    r.count = int(sel_fluid.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_fluid(sel_fluid[k]);
    return r;
  }
  G_boundary mk_boundary(Group *grp) const {
    G_boundary r{};
    r.n = uint32_t(grp->count);
    r.index = grp->index;
    VaryingField &f_x = grp->varying.at("position");
    r.v_x = static_cast<float4 *>(f_x.d);
    VaryingField &f_V = grp->varying.at("volume");
    r.v_V = static_cast<float *>(f_V.d);
    r.u_mu = SReal{static_cast<float *>(model_->small_ptr(grp->uniform.at("dynamic_viscosity")))};
    return r;
  }
  G_boundary_all all_boundary() const {
    G_boundary_all r{};
    r.count = int(sel_boundary.size());
    for (int k = 0; k < r.count; ++k) r.g[k] = mk_boundary(sel_boundary[k]);
    return r;
  }
  void proc_compute_diagonal(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // foreach fluid particle f
      for (Group *pg : sel_fluid) {
        if (pg->count == 0) continue;
        uint32_t blocks_ = uint32_t((pg->count + kGenNT - 1) / kGenNT);
        NbrView const &lv_ = nh.lists(pg->index, s);
        k_compute_diagonal_p0<<<blocks_, kGenNT, 0, s>>>(mk_fluid(pg), all_boundary(), glob(), lv_, frame_, nullptr, 0u, 0u);
        count_launch();
      }
      for (Group *pg : sel_fluid) pg->varying.at("wkbb18_system_diagonal").version++;
    }
    PG_LAUNCH_CHECK();
  }
  void proc_accumulate_acceleration(Nhood &nh, cudaStream_t s) {
    (void)nh;
    { // solve pcg real[] over fluid particle f
      for (Group *pg : sel_fluid) {
        G_fluid pp_ = mk_fluid(pg);
        uint32_t n_ = uint32_t(pg->count);
        if (n_ == 0) { k_pcg_zero<<<1, 1, 0, s>>>(pp_.u_pcg_iterations); count_launch(); continue; }
        uint32_t nb_ = (n_ + kGenNT - 1) / kGenNT;
        ensure_pcg(n_ * sizeof(float4), nb_);
        float4 *x_ = pcg_vec<float4>(0, n_), *b_ = pcg_vec<float4>(1, n_), *r_ = pcg_vec<float4>(2, n_);
        float4 *p_ = pcg_vec<float4>(3, n_), *q_ = pcg_vec<float4>(4, n_), *y_ = pcg_vec<float4>(5, n_);
        double *c0_ = pcg_part_, *c1_ = pcg_part_ + pcg_part_cap_, *c2_ = pcg_part_ + 2 * pcg_part_cap_;
        NbrView const &lv_ = nh.lists(pg->index, s);
        float4 *none_ = nullptr;
        k_accumulate_acceleration_v0_guess<<<nb_, kGenNT, 0, s>>>(pp_, glob(), lv_, frame_, x_, none_);
        k_accumulate_acceleration_v0_right_hand_side<<<nb_, kGenNT, 0, s>>>(pp_, all_boundary(), glob(), lv_, frame_, b_, none_);
        k_accumulate_acceleration_v0_system<<<nb_, kGenNT, 0, s>>>(pp_, all_boundary(), glob(), lv_, frame_, r_, x_);
        k_pcg_residual<float4><<<nb_, kPcgNT, 0, s>>>(n_, r_, b_, c0_);
        k_accumulate_acceleration_v0_preconditioner<<<nb_, kGenNT, 0, s>>>(pp_, glob(), lv_, frame_, y_, r_);
        k_pcg_start<float4><<<nb_, kPcgNT, 0, s>>>(n_, p_, y_, r_, c1_, c2_);
        k_pcg_begin<<<1, 1, 0, s>>>(pcg_state_, pp_.u_pcg_max_error, pp_.u_pcg_max_iters, c0_, c1_, c2_, nb_);
        for (int k = 0; k < 7; ++k) count_launch();
        for (long it_ = 0;; ++it_) {
          // q = A p; alpha; x += alpha p, r += alpha q; y = T r; beta; p = -y + beta p
          k_accumulate_acceleration_v0_system<<<nb_, kGenNT, 0, s>>>(pp_, all_boundary(), glob(), lv_, frame_, q_, p_);
          k_pcg_dot<float4><<<nb_, kPcgNT, 0, s>>>(n_, p_, q_, c0_);
          k_pcg_step<<<1, 1, 0, s>>>(pcg_state_, c0_, nb_);
          k_pcg_update<float4><<<nb_, kPcgNT, 0, s>>>(n_, x_, r_, p_, q_, pcg_state_, c1_);
          k_accumulate_acceleration_v0_preconditioner<<<nb_, kGenNT, 0, s>>>(pp_, glob(), lv_, frame_, y_, r_);
          k_pcg_dot<float4><<<nb_, kPcgNT, 0, s>>>(n_, r_, y_, c2_);
          k_pcg_next<<<1, 1, 0, s>>>(pcg_state_, c1_, c2_, nb_);
          k_pcg_direction<float4><<<nb_, kPcgNT, 0, s>>>(n_, p_, y_, pcg_state_);
          for (int k = 0; k < 8; ++k) count_launch();
          PG_CUDA(cudaMemcpyAsync(pcg_stop_h_, &pcg_state_->stop, sizeof(int), cudaMemcpyDeviceToHost, s));
          PG_CUDA(cudaStreamSynchronize(s));
          if (*pcg_stop_h_) break;
          if (it_ > (1L << 30)) throw Error("solve pcg did not stop");
        }
        k_accumulate_acceleration_v0_apply<<<nb_, kGenNT, 0, s>>>(pp_, glob(), lv_, frame_, none_, x_);
        k_pcg_end<<<1, 1, 0, s>>>(pcg_state_, pp_.u_pcg_iterations);
        count_launch();
        count_launch();
      }
      for (Group *pg : sel_fluid) pg->varying.at("wkbb18_velocity_delta").version++;
      for (Group *pg : sel_fluid) pg->varying.at("acceleration").version++;
    }
    PG_LAUNCH_CHECK();
  }
};

} // namespace gen_wkbb18_1c18b6a3b4c9
} // namespace prtcl_gpu

extern "C" void prtcl_gpu_plugin_init() {
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_aiast12[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_aiast12_137ff5928731::Scheme_());
  });
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_density[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_density_51043b23b2ed::Scheme_());
  });
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_gravity[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_gravity_20408f2f18b0::Scheme_());
  });
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_iisph[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_iisph_177f18681cf7::Scheme_());
  });
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_symplectic_euler[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_symplectic_euler_13eb52a9f28b::Scheme_());
  });
  ::prtcl_gpu::register_scheme("prtcl::schemes::ref_wkbb18[T=f32, N=3, K=Cubic Spline]", [] {
    return std::unique_ptr<::prtcl_gpu::Scheme>(new ::prtcl_gpu::gen_wkbb18_1c18b6a3b4c9::Scheme_());
  });
}
