// Model archives in the reference's native binary format, so that model
// states written by prtcl (model.N.bin) load straight onto the device and
// device states can be compared with the reference's outside this library.
//
// Format (util/archive.cpp:5-40 with the model's Save / Load,
// data/model.cpp:54-75): sizes are native size_t (8 bytes, little-endian on
// the supported hosts), strings are a size and the bytes, values are written
// component by component in the item layout (matrices column-major).
//   model    : globals (a uniform manager), group count, then per group
//              name, type and the group
//   group    : tag count, tags, varying manager, uniform manager
//              (data/group.cpp:31-59)
//   varying  : item count, field count, then per field name, tensor type,
//              item count and count x components values
//              (data/varying_manager.cpp:21-45)
//   uniform  : field count, then per field name, tensor type and the
//              components (data/uniform_manager.cpp:22-40)
//   tensor type: component type name ("b", "s32", "s64", "f32", "f64"),
//              rank, extents (data/tensor_type.cpp:7-15, data/shape.cpp:9-19,
//              data/component_type.cpp:15-38)
// The device model holds f32 and s32 components of rank <= 2; archives with
// other component types are refused.
#include "model.hpp"

#include <cstdio>
#include <cstring>
#include <vector>

namespace prtcl_gpu {

namespace {

constexpr uint64_t kMaxString = uint64_t(1) << 20;
constexpr uint64_t kMaxItems = uint64_t(1) << 34;

class Writer {
public:
  explicit Writer(std::string const &path) : f_(std::fopen(path.c_str(), "wb")) {
    if (!f_) throw Error("archive: cannot write " + path);
  }
  ~Writer() {
    if (f_) std::fclose(f_);
  }
  void size(uint64_t v) { bytes(&v, sizeof v); }
  void str(std::string const &s) {
    size(s.size());
    bytes(s.data(), s.size());
  }
  void bytes(void const *p, size_t n) {
    if (n && std::fwrite(p, 1, n, f_) != n) throw Error("archive: write failed");
  }
  void close() {
    if (std::fclose(f_) != 0) {
      f_ = nullptr;
      throw Error("archive: write failed");
    }
    f_ = nullptr;
  }

private:
  std::FILE *f_;
};

class Reader {
public:
  explicit Reader(std::string const &path) : f_(std::fopen(path.c_str(), "rb")) {
    if (!f_) throw Error("archive: cannot read " + path);
  }
  ~Reader() { std::fclose(f_); }
  uint64_t size() {
    uint64_t v = 0;
    bytes(&v, sizeof v);
    return v;
  }
  std::string str() {
    uint64_t n = size();
    if (n > kMaxString) throw Error("archive: string of " + std::to_string(n) + " bytes (corrupt archive?)");
    std::string s(size_t(n), '\0');
    bytes(s.data(), s.size());
    return s;
  }
  void bytes(void *p, size_t n) {
    if (n && std::fread(p, 1, n, f_) != n) throw Error("archive: truncated");
  }
  bool at_end() { return std::fgetc(f_) == EOF; }

private:
  std::FILE *f_;
};

void save_type(Writer &w, FieldType const &t) {
  w.str(t.ctype == CType::F32 ? "f32" : "s32");
  w.size(uint64_t(t.rank));
  for (int r = 0; r < t.rank; ++r) w.size(uint64_t(t.ext[r]));
}

FieldType load_type(Reader &r, std::string const &what) {
  std::string c = r.str();
  FieldType t;
  if (c == "f32") t.ctype = CType::F32;
  else if (c == "s32") t.ctype = CType::I32;
  else
    throw Error("archive: " + what + " has component type '" + c +
                "'; the device model holds f32 and s32 components");
  uint64_t rank = r.size();
  if (rank > 2) throw Error("archive: " + what + " has rank " + std::to_string(rank) + " (at most 2)");
  t.rank = int(rank);
  for (uint64_t k = 0; k < rank; ++k) {
    uint64_t e = r.size();
    if (e == 0 || e > 1024) throw Error("archive: " + what + " has extent " + std::to_string(e));
    t.ext[k] = int(e);
  }
  return t;
}

void save_small(Writer &w, Model &m, std::map<std::string, SmallField> const &fields, cudaStream_t s) {
  w.size(fields.size());
  for (auto const &kv : fields) {
    w.str(kv.first);
    save_type(w, kv.second.type);
    std::vector<uint32_t> v(kv.second.type.comps());
    m.small_get(kv.second, v.data(), s);
    w.bytes(v.data(), v.size() * 4);
  }
}

} // namespace

void save_model(Model &m, std::string const &path, cudaStream_t s) {
  Writer w(path);
  save_small(w, m, m.globals(), s);
  auto groups = m.groups_by_index(); // alphabetical, as the reference's map
  w.size(groups.size());
  for (Group *g : groups) {
    w.str(g->name);
    w.str(g->type);
    w.size(g->tags.size());
    for (auto const &t : g->tags) w.str(t);
    w.size(g->count);
    w.size(g->varying.size());
    std::vector<uint32_t> buf;
    for (auto const &kv : g->varying) {
      w.str(kv.first);
      save_type(w, kv.second.type);
      w.size(g->count);
      buf.resize(g->count * kv.second.type.comps());
      download_varying(kv.second, g->count, buf.data(), g->count, s);
      w.bytes(buf.data(), buf.size() * 4);
    }
    save_small(w, m, g->uniform, s);
  }
  w.close();
}

void load_model(Model &m, std::string const &path, cudaStream_t s) {
  Reader r(path);
  uint64_t ng = r.size();
  // globals
  for (uint64_t k = 0; k < ng; ++k) {
    std::string name = r.str();
    FieldType t = load_type(r, "global field '" + name + "'");
    std::vector<uint32_t> v(t.comps());
    r.bytes(v.data(), v.size() * 4);
    m.small_set(m.add_global(name, t), v.data(), s);
  }
  uint64_t groups = r.size();
  if (groups > 4096) throw Error("archive: " + std::to_string(groups) + " groups (corrupt archive?)");
  for (uint64_t gi = 0; gi < groups; ++gi) {
    std::string name = r.str(), type = r.str();
    Group &g = m.add_group(name, type);
    if (g.type != type) throw Error("archive: group '" + name + "' exists with type '" + g.type + "'");
    uint64_t tags = r.size();
    if (tags > 4096) throw Error("archive: " + std::to_string(tags) + " tags (corrupt archive?)");
    for (uint64_t k = 0; k < tags; ++k) g.tags.insert(r.str());
    uint64_t count = r.size();
    if (count > kMaxItems) throw Error("archive: " + std::to_string(count) + " items (corrupt archive?)");
    g.resize(size_t(count), s);
    uint64_t nf = r.size();
    if (nf > 4096) throw Error("archive: " + std::to_string(nf) + " fields (corrupt archive?)");
    std::vector<uint32_t> buf;
    for (uint64_t k = 0; k < nf; ++k) {
      std::string fname = r.str();
      FieldType t = load_type(r, "field '" + name + "." + fname + "'");
      uint64_t n = r.size();
      if (n != count)
        throw Error("archive: field '" + name + "." + fname + "' has " + std::to_string(n) + " items, the group " +
                    std::to_string(count));
      VaryingField &f = g.add_varying(fname, t);
      buf.resize(size_t(n) * t.comps());
      r.bytes(buf.data(), buf.size() * 4);
      upload_varying(f, g.count, buf.data(), size_t(n), s, true);
    }
    uint64_t nu = r.size();
    if (nu > 4096) throw Error("archive: " + std::to_string(nu) + " uniform fields (corrupt archive?)");
    for (uint64_t k = 0; k < nu; ++k) {
      std::string uname = r.str();
      FieldType t = load_type(r, "uniform field '" + name + "." + uname + "'");
      std::vector<uint32_t> v(t.comps());
      r.bytes(v.data(), v.size() * 4);
      m.small_set(g.add_uniform(uname, t), v.data(), s);
    }
  }
  if (!r.at_end()) throw Error("archive: trailing bytes after the model");
  m.layout_version++;
}

} // namespace prtcl_gpu
