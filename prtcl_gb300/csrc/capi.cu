// extern "C" surface of the library (include/prtcl_gpu.h).
#include "../../include/prtcl_gpu.h"
#include "batch.hpp"
#include "schemes.hpp"
#include "server.hpp"

#include <atomic>
#include <dlfcn.h>
#include <cstdio>
#include <cstring>
#include <string>

using namespace prtcl_gpu;

struct prtcl_gpu_model {
  Model m;
};
struct prtcl_gpu_nhood {
  Nhood n;
};
struct prtcl_gpu_scheme {
  std::unique_ptr<Scheme> s;
};
struct prtcl_gpu_batch {
  std::unique_ptr<Batch> b;
};
struct prtcl_gpu_server {
  std::unique_ptr<Server> s;
};

namespace prtcl_gpu {
static std::atomic<uint64_t> g_launches{0};
void count_launch() { g_launches.fetch_add(1, std::memory_order_relaxed); }
void uncount_launches(uint64_t n) { g_launches.fetch_sub(n, std::memory_order_relaxed); }
uint64_t launch_count() { return g_launches.load(std::memory_order_relaxed); }
} // namespace prtcl_gpu

namespace {

thread_local std::string g_last_error;

struct NotFound : Error {
  using Error::Error;
};

int fail(int code, std::string const &msg) {
  g_last_error = msg;
  return code;
}

template <class F> int guard(F &&f) {
  try {
    f();
    return PRTCL_GPU_OK;
  } catch (NotFound const &e) {
    return fail(PRTCL_GPU_NOT_FOUND, e.what());
  } catch (std::exception const &e) {
    std::string w = e.what();
    if (w == "procedure does not exist" || w == "scheme is not registered" ||
        w.rfind("group does not exist", 0) == 0 || w.rfind("field does not exist", 0) == 0)
      return fail(PRTCL_GPU_NOT_FOUND, w);
    return fail(PRTCL_GPU_ERROR, w);
  } catch (...) {
    return fail(PRTCL_GPU_ERROR, "unknown error");
  }
}

#define NEED(p)                                                                                        \
  do {                                                                                                 \
    if (!(p)) return fail(PRTCL_GPU_INVALID, std::string("invalid argument: ") + #p + " is null");     \
  } while (0)

FieldType ftype(char const *ctype, int32_t rank, int32_t const *ext) {
  int e[2] = {1, 1};
  for (int r = 0; r < rank && r < 2; ++r) e[r] = ext ? ext[r] : 0;
  return parse_field_type(ctype, rank, e);
}

VaryingField &varying(Model &m, char const *group, char const *field) {
  Group &g = m.group(group);
  VaryingField *f = g.find_varying(field);
  if (!f) throw NotFound(std::string("field does not exist: ") + group + "." + field);
  return *f;
}

SmallField &uniform(Model &m, char const *group, char const *field) {
  Group &g = m.group(group);
  auto it = g.uniform.find(field);
  if (it == g.uniform.end()) throw NotFound(std::string("field does not exist: ") + group + "." + field);
  return it->second;
}

SmallField &global(Model &m, char const *field) {
  SmallField *f = m.find_global(field);
  if (!f) throw NotFound(std::string("field does not exist: global.") + field);
  return *f;
}

int write_str(std::string const &s, char *buf, int64_t size, int64_t *needed) {
  if (needed) *needed = int64_t(s.size()) + 1;
  if (buf && size > 0) {
    size_t n = std::min<size_t>(s.size(), size_t(size - 1));
    std::memcpy(buf, s.data(), n);
    buf[n] = '\0';
  }
  return PRTCL_GPU_OK;
}

std::string join(std::vector<std::string> const &v) {
  std::string r;
  for (size_t i = 0; i < v.size(); ++i) r += (i ? "\n" : "") + v[i];
  return r;
}

} // namespace

extern "C" {

const char *prtcl_gpu_last_error(void) { return g_last_error.c_str(); }
const char *prtcl_gpu_version(void) { return "prtcl_gb300 0.1 (sm_103a)"; }
uint64_t prtcl_gpu_launch_count(void) { return launch_count() + device_loop_kernels(); }

int prtcl_gpu_model_create(prtcl_gpu_model **out) {
  NEED(out);
  return guard([&] {
    // the no-alloc upload's staging array and kernels are made resident now,
    // before a host can hand the rest of the device memory to its own pool
    noalloc_prepare();
    *out = new prtcl_gpu_model();
  });
}
int prtcl_gpu_model_destroy(prtcl_gpu_model *model) {
  return guard([&] { delete model; });
}
int prtcl_gpu_group_add(prtcl_gpu_model *model, const char *name, const char *type) {
  NEED(model);
  NEED(name);
  NEED(type);
  return guard([&] { model->m.add_group(name, type); });
}
int prtcl_gpu_group_add_tag(prtcl_gpu_model *model, const char *group, const char *tag) {
  NEED(model);
  NEED(group);
  NEED(tag);
  return guard([&] { model->m.group(group).tags.insert(tag); });
}
int prtcl_gpu_group_resize(prtcl_gpu_model *model, const char *group, int64_t count) {
  NEED(model);
  NEED(group);
  if (count < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative count");
  return guard([&] {
    model->m.group(group).resize(size_t(count), model->m.stream());
    PG_CUDA(cudaStreamSynchronize(model->m.stream()));
  });
}
int prtcl_gpu_group_count(prtcl_gpu_model *model, const char *group, int64_t *count_out) {
  NEED(model);
  NEED(group);
  NEED(count_out);
  return guard([&] { *count_out = int64_t(model->m.group(group).count); });
}
int prtcl_gpu_group_index(prtcl_gpu_model *model, const char *group, int32_t *index_out) {
  NEED(model);
  NEED(group);
  NEED(index_out);
  return guard([&] { *index_out = model->m.group(group).index; });
}
int prtcl_gpu_model_group_count(prtcl_gpu_model *model, int32_t *count_out) {
  NEED(model);
  NEED(count_out);
  return guard([&] { *count_out = int32_t(model->m.group_count()); });
}

int prtcl_gpu_field_add(prtcl_gpu_model *model, const char *group, const char *field, const char *ctype, int32_t rank,
                        const int32_t *extents) {
  NEED(model);
  NEED(group);
  NEED(field);
  return guard([&] {
    model->m.group(group).add_varying(field, ftype(ctype, rank, extents));
    PG_CUDA(cudaStreamSynchronize(model->m.stream()));
  });
}
int prtcl_gpu_field_upload(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                           int64_t count, void *stream) {
  NEED(model);
  NEED(group);
  NEED(field);
  if (count > 0) NEED(host);
  return guard([&] {
    Group &g = model->m.group(group);
    upload_varying(varying(model->m, group, field), g.count, host, size_t(count), model->m.pick(stream), true);
  });
}
int prtcl_gpu_field_upload_async(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                                 int64_t count, void *stream) {
  NEED(model);
  NEED(group);
  NEED(field);
  if (count > 0) NEED(host);
  return guard([&] {
    Group &g = model->m.group(group);
    upload_varying(varying(model->m, group, field), g.count, host, size_t(count), model->m.pick(stream), false);
  });
}
int prtcl_gpu_field_upload_noalloc(prtcl_gpu_model *model, const char *group, const char *field, const void *host,
                                   int64_t count, void *stream) {
  NEED(model);
  NEED(group);
  NEED(field);
  if (count > 0) NEED(host);
  return guard([&] {
    Group &g = model->m.group(group);
    upload_varying_noalloc(varying(model->m, group, field), g.count, host, size_t(count), model->m.pick(stream));
  });
}
int prtcl_gpu_field_download(prtcl_gpu_model *model, const char *group, const char *field, void *host, int64_t count,
                             void *stream) {
  NEED(model);
  NEED(group);
  NEED(field);
  if (count > 0) NEED(host);
  return guard([&] {
    Group &g = model->m.group(group);
    download_varying(varying(model->m, group, field), g.count, host, size_t(count), model->m.pick(stream));
  });
}
int prtcl_gpu_field_info(prtcl_gpu_model *model, const char *group, const char *field, char *ctype_out,
                         int32_t *rank_out, int32_t *extents_out) {
  NEED(model);
  NEED(group);
  NEED(field);
  return guard([&] {
    FieldType t = varying(model->m, group, field).type;
    if (ctype_out) std::strcpy(ctype_out, t.ctype == CType::F32 ? "f32" : "i32");
    if (rank_out) *rank_out = t.rank;
    if (extents_out) {
      extents_out[0] = t.ext[0];
      extents_out[1] = t.ext[1];
    }
  });
}

int prtcl_gpu_uniform_add(prtcl_gpu_model *model, const char *group, const char *field, const char *ctype,
                          int32_t rank, const int32_t *extents) {
  NEED(model);
  NEED(group);
  NEED(field);
  return guard([&] { model->m.group(group).add_uniform(field, ftype(ctype, rank, extents)); });
}
int prtcl_gpu_uniform_set(prtcl_gpu_model *model, const char *group, const char *field, const void *value) {
  NEED(model);
  NEED(group);
  NEED(field);
  NEED(value);
  return guard([&] { model->m.small_set(uniform(model->m, group, field), value, model->m.stream()); });
}
int prtcl_gpu_uniform_get(prtcl_gpu_model *model, const char *group, const char *field, void *value) {
  NEED(model);
  NEED(group);
  NEED(field);
  NEED(value);
  return guard([&] { model->m.small_get(uniform(model->m, group, field), value, model->m.stream()); });
}
int prtcl_gpu_global_add(prtcl_gpu_model *model, const char *field, const char *ctype, int32_t rank,
                         const int32_t *extents) {
  NEED(model);
  NEED(field);
  return guard([&] { model->m.add_global(field, ftype(ctype, rank, extents)); });
}
int prtcl_gpu_global_set(prtcl_gpu_model *model, const char *field, const void *value) {
  NEED(model);
  NEED(field);
  NEED(value);
  return guard([&] { model->m.small_set(global(model->m, field), value, model->m.stream()); });
}
int prtcl_gpu_global_set_async(prtcl_gpu_model *model, const char *field, const void *value, void *stream) {
  NEED(model);
  NEED(field);
  NEED(value);
  return guard([&] { model->m.small_set_async(global(model->m, field), value, model->m.pick(stream)); });
}
int prtcl_gpu_model_stats(prtcl_gpu_model *model, double *out, int32_t n, int32_t reset) {
  NEED(model);
  if (n > 0) NEED(out);
  return guard([&] {
    double st[16];
    PG_CUDA(cudaMemcpyAsync(st, model->m.stats_d, sizeof st, cudaMemcpyDeviceToHost, model->m.stream()));
    PG_CUDA(cudaStreamSynchronize(model->m.stream()));
    for (int i = 0; i < n && i < 16; ++i) out[i] = st[i];
    if (reset) model->m.stats_reset(model->m.stream());
  });
}
int prtcl_gpu_global_get(prtcl_gpu_model *model, const char *field, void *value) {
  NEED(model);
  NEED(field);
  NEED(value);
  return guard([&] { model->m.small_get(global(model->m, field), value, model->m.stream()); });
}
static void write_type(FieldType const &t, char *ctype_out, int32_t *rank_out, int32_t *extents_out) {
  if (ctype_out) std::strcpy(ctype_out, t.ctype == CType::F32 ? "f32" : "i32");
  if (rank_out) *rank_out = t.rank;
  if (extents_out) {
    extents_out[0] = t.ext[0];
    extents_out[1] = t.ext[1];
  }
}
int prtcl_gpu_uniform_info(prtcl_gpu_model *model, const char *group, const char *field, char *ctype_out,
                           int32_t *rank_out, int32_t *extents_out) {
  NEED(model);
  NEED(group);
  NEED(field);
  return guard([&] { write_type(uniform(model->m, group, field).type, ctype_out, rank_out, extents_out); });
}
int prtcl_gpu_global_info(prtcl_gpu_model *model, const char *field, char *ctype_out, int32_t *rank_out,
                          int32_t *extents_out) {
  NEED(model);
  NEED(field);
  return guard([&] { write_type(global(model->m, field).type, ctype_out, rank_out, extents_out); });
}
int prtcl_gpu_model_stream(prtcl_gpu_model *model, void **stream_out) {
  NEED(model);
  NEED(stream_out);
  *stream_out = static_cast<void *>(model->m.stream());
  return PRTCL_GPU_OK;
}
int prtcl_gpu_model_synchronize(prtcl_gpu_model *model, void *stream) {
  NEED(model);
  return guard([&] {
    if (stream) PG_CUDA(cudaStreamSynchronize(static_cast<cudaStream_t>(stream)));
    PG_CUDA(cudaStreamSynchronize(model->m.stream()));
  });
}

int prtcl_gpu_model_group_names(prtcl_gpu_model *model, char *buf, int64_t size, int64_t *needed_out) {
  NEED(model);
  std::vector<std::string> names;
  for (Group *g : model->m.groups_by_index()) names.push_back(g->name);
  return write_str(join(names), buf, size, needed_out);
}
int prtcl_gpu_group_save_vtk(prtcl_gpu_model *model, const char *group, const char *path) {
  NEED(model);
  NEED(group);
  NEED(path);
  return guard([&] { save_vtk(model->m.group(group), path, model->m.stream()); });
}
int prtcl_gpu_model_save(prtcl_gpu_model *model, const char *path) {
  NEED(model);
  NEED(path);
  return guard([&] { save_model(model->m, path, model->m.stream()); });
}
int prtcl_gpu_model_load(prtcl_gpu_model *model, const char *path) {
  NEED(model);
  NEED(path);
  return guard([&] { load_model(model->m, path, model->m.stream()); });
}
int prtcl_gpu_profile_enable(prtcl_gpu_model *model, int32_t enable) {
  NEED(model);
  return guard([&] { model->m.prof.enabled = enable != 0; });
}
int prtcl_gpu_profile_read(prtcl_gpu_model *model, char *buf, int64_t size, int64_t *needed_out) {
  NEED(model);
  std::string text;
  int rc = guard([&] {
    for (auto &kv : model->m.prof.read()) {
      char line[256];
      std::snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), kv.second.count, kv.second.ms);
      text += line;
    }
  });
  if (rc != PRTCL_GPU_OK) return rc;
  return write_str(text, buf, size, needed_out);
}
int prtcl_gpu_profile_reset(prtcl_gpu_model *model) {
  NEED(model);
  return guard([&] { model->m.prof.reset(); });
}

namespace {
int tune_set(Model &m, const char *knob, int32_t value) {
  int k = tune_knob_find(knob);
  if (k < 0) return fail(PRTCL_GPU_NOT_FOUND, std::string("unknown tuning knob: ") + knob);
  if (!tune_value_ok(k, value))
    return fail(PRTCL_GPU_INVALID, "invalid argument: value " + std::to_string(value) + " for knob " + knob);
  m.tune.v[k] = value;
  return PRTCL_GPU_OK;
}
int tune_get(Model &m, const char *knob, int32_t *value_out) {
  int k = tune_knob_find(knob);
  if (k < 0) return fail(PRTCL_GPU_NOT_FOUND, std::string("unknown tuning knob: ") + knob);
  *value_out = m.tune.v[k];
  return PRTCL_GPU_OK;
}
} // namespace

int prtcl_gpu_tune_knobs(char *buf, int64_t size, int64_t *needed_out) {
  return write_str(tune_knob_table(), buf, size, needed_out);
}
int prtcl_gpu_model_tune_set(prtcl_gpu_model *model, const char *knob, int32_t value) {
  NEED(model);
  NEED(knob);
  return tune_set(model->m, knob, value);
}
int prtcl_gpu_model_tune_get(prtcl_gpu_model *model, const char *knob, int32_t *value_out) {
  NEED(model);
  NEED(knob);
  NEED(value_out);
  return tune_get(model->m, knob, value_out);
}

int prtcl_gpu_nhood_create(prtcl_gpu_nhood **out) {
  NEED(out);
  return guard([&] { *out = new prtcl_gpu_nhood(); });
}
int prtcl_gpu_nhood_destroy(prtcl_gpu_nhood *nhood) {
  return guard([&] { delete nhood; });
}
int prtcl_gpu_nhood_set_radius(prtcl_gpu_nhood *nhood, double radius) {
  NEED(nhood);
  if (!(radius > 0)) return fail(PRTCL_GPU_INVALID, "invalid argument: radius must be positive");
  return guard([&] { nhood->n.set_radius(radius); });
}
int prtcl_gpu_nhood_load(prtcl_gpu_nhood *nhood, prtcl_gpu_model *model) {
  NEED(nhood);
  NEED(model);
  return guard([&] { nhood->n.load(model->m); });
}
int prtcl_gpu_nhood_update(prtcl_gpu_nhood *nhood, void *stream) {
  NEED(nhood);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood::Update before Load");
    nhood->n.update(nhood->n.model()->pick(stream));
  });
}
int prtcl_gpu_nhood_query(prtcl_gpu_nhood *nhood, int32_t query_group, int64_t *pairs_out, void *stream) {
  NEED(nhood);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood::Query before Load");
    cudaStream_t s = nhood->n.model()->pick(stream);
    if (pairs_out) *pairs_out = int64_t(nhood->n.pair_count(query_group, s));
    else nhood->n.lists(query_group, s);
  });
}
int prtcl_gpu_nhood_permute(prtcl_gpu_nhood *nhood, prtcl_gpu_model *model, void *stream) {
  NEED(nhood);
  NEED(model);
  return guard([&] { nhood->n.permute(model->m, model->m.pick(stream)); });
}
int prtcl_gpu_nhood_copy_neighbors(prtcl_gpu_nhood *nhood, int32_t group, int64_t index, int64_t *counts_out,
                                   int64_t *indices_out, int64_t capacity, int64_t *total_out) {
  NEED(nhood);
  NEED(counts_out);
  if (capacity > 0) NEED(indices_out);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood::CopyNeighbors before Load");
    size_t k = nhood->n.copy_neighbors(group, size_t(index), counts_out, indices_out, size_t(capacity),
                                       nhood->n.model()->stream());
    if (total_out) *total_out = int64_t(k);
  });
}
int prtcl_gpu_nhood_copy_lists(prtcl_gpu_nhood *nhood, int32_t query_group, int32_t neighbor_group,
                               int64_t *offsets_out, uint32_t *indices_out, int64_t capacity) {
  NEED(nhood);
  NEED(offsets_out);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood not loaded");
    nhood->n.copy_lists(query_group, neighbor_group, offsets_out, indices_out, size_t(capacity),
                        nhood->n.model()->stream());
  });
}
int prtcl_gpu_nhood_staged_tiles(prtcl_gpu_nhood *nhood, int32_t query_group, int64_t *staged_out,
                                 int64_t *tiles_out) {
  NEED(nhood);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood not loaded");
    size_t tiles = 0;
    size_t k = nhood->n.staged_tiles(query_group, tiles, nhood->n.model()->stream());
    if (staged_out) *staged_out = int64_t(k);
    if (tiles_out) *tiles_out = int64_t(tiles);
  });
}
int prtcl_gpu_nhood_grid_size(prtcl_gpu_nhood *nhood, int64_t *sorted_count_out, int64_t *cell_count_out) {
  NEED(nhood);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood not loaded");
    if (sorted_count_out) *sorted_count_out = int64_t(nhood->n.sorted_count());
    if (cell_count_out) *cell_count_out = int64_t(nhood->n.cell_count(nhood->n.model()->stream()));
  });
}
int prtcl_gpu_nhood_copy_grid(prtcl_gpu_nhood *nhood, uint32_t *sorted_out, int32_t *cell_grid_index_out,
                              int32_t *cell_range_out, int32_t *cell_adjacency_out) {
  NEED(nhood);
  return guard([&] {
    if (!nhood->n.loaded()) throw Error("Neighborhood not loaded");
    nhood->n.copy_grid(sorted_out, cell_grid_index_out, cell_range_out, cell_adjacency_out, nhood->n.model()->stream());
  });
}

int prtcl_gpu_scheme_new(const char *full_name, prtcl_gpu_scheme **out) {
  NEED(full_name);
  NEED(out);
  return guard([&] {
    auto s = new_scheme(full_name);
    *out = new prtcl_gpu_scheme{std::move(s)};
  });
}
int prtcl_gpu_scheme_destroy(prtcl_gpu_scheme *scheme) {
  return guard([&] { delete scheme; });
}
int prtcl_gpu_scheme_load(prtcl_gpu_scheme *scheme, prtcl_gpu_model *model) {
  NEED(scheme);
  NEED(model);
  return guard([&] {
    scheme->s->load(model->m);
    PG_CUDA(cudaStreamSynchronize(model->m.stream()));
  });
}
int prtcl_gpu_scheme_run(prtcl_gpu_scheme *scheme, const char *procedure, prtcl_gpu_nhood *nhood, void *stream) {
  NEED(scheme);
  NEED(procedure);
  NEED(nhood);
  return guard([&] {
    Model *m = scheme->s->model();
    scheme->s->run(procedure, nhood->n, m ? m->pick(stream) : static_cast<cudaStream_t>(stream));
  });
}
int prtcl_gpu_scheme_full_name(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out) {
  NEED(scheme);
  return write_str(scheme->s->full_name(), buf, size, needed_out);
}
int prtcl_gpu_scheme_procedure_names(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out) {
  NEED(scheme);
  return write_str(join(scheme->s->procedure_names()), buf, size, needed_out);
}
int prtcl_gpu_scheme_source(prtcl_gpu_scheme *scheme, char *buf, int64_t size, int64_t *needed_out) {
  NEED(scheme);
  return write_str(scheme->s->source(), buf, size, needed_out);
}
int prtcl_gpu_registry_scheme_names(char *buf, int64_t size, int64_t *needed_out) {
  return write_str(join(scheme_names()), buf, size, needed_out);
}
int prtcl_gpu_scheme_load_plugin(const char *path) {
  NEED(path);
  return guard([&] {
    // kept open for the life of the process: the schemes it registered
    // point into it
    void *h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
    if (!h) throw Error(std::string("cannot load scheme plugin: ") + dlerror());
    auto init = reinterpret_cast<void (*)()>(dlsym(h, "prtcl_gpu_plugin_init"));
    if (!init) throw Error("scheme plugin has no prtcl_gpu_plugin_init: " + std::string(path));
    init();
  });
}

// ---- batched scenes ----

int prtcl_gpu_batch_create(const prtcl_gpu_batch_params *params, prtcl_gpu_batch **out) {
  NEED(params);
  NEED(out);
  *out = nullptr;
  return guard([&] {
    auto b = std::make_unique<prtcl_gpu_batch>();
    b->b = std::make_unique<Batch>(*params);
    *out = b.release();
  });
}
int prtcl_gpu_batch_destroy(prtcl_gpu_batch *batch) {
  delete batch;
  return PRTCL_GPU_OK;
}
int prtcl_gpu_batch_add_scene(prtcl_gpu_batch *batch, const float *fluid_xyz, int64_t fluid_count,
                              const float *boundary_xyz, int64_t boundary_count, int64_t *scene_id_out) {
  NEED(batch);
  NEED(scene_id_out);
  if (fluid_count < 0 || boundary_count < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative count");
  return guard([&] {
    *scene_id_out = batch->b->add(fluid_xyz, size_t(fluid_count), boundary_xyz, size_t(boundary_count));
  });
}
int prtcl_gpu_batch_remove_scene(prtcl_gpu_batch *batch, int64_t scene_id) {
  NEED(batch);
  return guard([&] { batch->b->remove(scene_id); });
}
int prtcl_gpu_batch_step(prtcl_gpu_batch *batch, int32_t steps) {
  NEED(batch);
  if (steps < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative step count");
  return guard([&] { batch->b->step(steps); });
}
int prtcl_gpu_batch_synchronize(prtcl_gpu_batch *batch) {
  NEED(batch);
  return guard([&] { batch->b->synchronize(); });
}
int prtcl_gpu_batch_scene_info(prtcl_gpu_batch *batch, int64_t scene_id, prtcl_gpu_scene_info *out) {
  NEED(batch);
  NEED(out);
  return guard([&] { *out = batch->b->info(scene_id); });
}
int prtcl_gpu_batch_download(prtcl_gpu_batch *batch, int64_t scene_id, const char *field, void *host, int64_t count) {
  NEED(batch);
  NEED(field);
  if (count > 0) NEED(host);
  if (count < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative count");
  return guard([&] { batch->b->download(scene_id, field, host, size_t(count)); });
}
int prtcl_gpu_batch_scene_count(prtcl_gpu_batch *batch, int32_t *count_out) {
  NEED(batch);
  NEED(count_out);
  return guard([&] { *count_out = int32_t(batch->b->scene_count()); });
}
int prtcl_gpu_batch_particles(prtcl_gpu_batch *batch, int64_t *fluid_out, int64_t *boundary_out) {
  NEED(batch);
  NEED(fluid_out);
  NEED(boundary_out);
  return guard([&] { batch->b->particles(*fluid_out, *boundary_out); });
}
int prtcl_gpu_batch_device_bytes(prtcl_gpu_batch *batch, int64_t *bytes_out) {
  NEED(batch);
  NEED(bytes_out);
  return guard([&] { *bytes_out = int64_t(batch->b->device_bytes()); });
}
int prtcl_gpu_batch_profile_enable(prtcl_gpu_batch *batch, int32_t enable) {
  NEED(batch);
  return guard([&] { batch->b->model().prof.enabled = enable != 0; });
}
int prtcl_gpu_batch_tune_set(prtcl_gpu_batch *batch, const char *knob, int32_t value) {
  NEED(batch);
  NEED(knob);
  return tune_set(batch->b->model(), knob, value);
}
int prtcl_gpu_batch_tune_get(prtcl_gpu_batch *batch, const char *knob, int32_t *value_out) {
  NEED(batch);
  NEED(knob);
  NEED(value_out);
  return tune_get(batch->b->model(), knob, value_out);
}
int prtcl_gpu_batch_profile_read(prtcl_gpu_batch *batch, char *buf, int64_t size, int64_t *needed_out) {
  NEED(batch);
  std::string text;
  int rc = guard([&] {
    for (auto &kv : batch->b->model().prof.read()) {
      char line[256];
      std::snprintf(line, sizeof line, "%s %lld %.6f\n", kv.first.c_str(), kv.second.count, kv.second.ms);
      text += line;
    }
  });
  if (rc != PRTCL_GPU_OK) return rc;
  return write_str(text, buf, size, needed_out);
}

int prtcl_gpu_server_create(const prtcl_gpu_batch_params *batch, const prtcl_gpu_server_params *params,
                            prtcl_gpu_server **out) {
  NEED(batch);
  NEED(params);
  NEED(out);
  *out = nullptr;
  return guard([&] {
    auto s = std::make_unique<prtcl_gpu_server>();
    s->s = std::make_unique<Server>(device_serve_batch(*batch), *params);
    *out = s.release();
  });
}
int prtcl_gpu_server_create_custom(const prtcl_gpu_server_batch_ops *ops, void *user,
                                   const prtcl_gpu_server_params *params, prtcl_gpu_server **out) {
  NEED(ops);
  NEED(params);
  NEED(out);
  *out = nullptr;
  return guard([&] {
    auto s = std::make_unique<prtcl_gpu_server>();
    s->s = std::make_unique<Server>(callback_serve_batch(*ops, user), *params);
    *out = s.release();
  });
}
int prtcl_gpu_server_destroy(prtcl_gpu_server *server) {
  delete server;
  return PRTCL_GPU_OK;
}
int prtcl_gpu_server_submit(prtcl_gpu_server *server, int64_t request_id, double arrival, const float *fluid_xyz,
                            int64_t fluid_count, const float *boundary_xyz, int64_t boundary_count, int64_t steps) {
  NEED(server);
  if (fluid_count < 0 || boundary_count < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative count");
  if (steps < 1) return fail(PRTCL_GPU_INVALID, "invalid argument: a request needs at least one step");
  return guard([&] {
    server->s->submit(request_id, arrival, fluid_xyz, size_t(fluid_count), boundary_xyz, size_t(boundary_count),
                      steps);
  });
}
int prtcl_gpu_server_turn(prtcl_gpu_server *server, int32_t *stepped_out) {
  NEED(server);
  return guard([&] {
    bool stepped = server->s->turn();
    if (stepped_out) *stepped_out = stepped ? 1 : 0;
  });
}
int prtcl_gpu_server_status_get(prtcl_gpu_server *server, prtcl_gpu_server_status *out) {
  NEED(server);
  NEED(out);
  return guard([&] { *out = server->s->status(); });
}
int prtcl_gpu_server_cancel(prtcl_gpu_server *server, int64_t request_id, int32_t *found_out) {
  NEED(server);
  NEED(found_out);
  return guard([&] { *found_out = server->s->cancel(request_id) ? 1 : 0; });
}
int prtcl_gpu_server_next_result(prtcl_gpu_server *server, prtcl_gpu_request_result *out, float *positions_xyz,
                                 int64_t capacity, int32_t *has_out) {
  NEED(server);
  NEED(out);
  NEED(has_out);
  if (capacity < 0) return fail(PRTCL_GPU_INVALID, "invalid argument: negative capacity");
  return guard([&] { *has_out = server->s->next_result(*out, positions_xyz, size_t(capacity)) ? 1 : 0; });
}

} // extern "C"
