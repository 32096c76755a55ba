// Device-resident mirror of prtcl's data model (data/model.cpp,
// data/group.hpp, data/varying_manager.hpp, data/uniform_manager.hpp).
//
// * Groups are ordered by name; a group's index is the alphabetical rank of
//   its name (data/model.cpp:26-31), so "b" (boundary) = 0, "f" (fluid) = 1.
// * Varying fields hold one value per item in HBM, one array per field:
//     real       -> float[count]
//     real[3]    -> float4[count]      (12-byte items padded to 16 bytes so a
//                                       gather is one aligned 16-byte load)
//     real[3][3] -> float[9][capacity] (planar, plane k = column-major index)
//     other      -> items back to back in the reference item layout
//   Upload and download convert from / to the reference's host layout (N
//   components contiguous per item, matrices column-major).
// * Uniform and global fields live in one device arena so kernels read them
//   from device memory: launches need no host round trip and can be captured
//   in CUDA graphs.
#pragma once

#include "common.cuh"
#include "profile.hpp"

#include <map>
#include <memory>
#include <set>
#include <string>
#include <vector>

namespace prtcl_gpu {

enum class CType : int { F32 = 0, I32 = 1 };

struct FieldType {
  CType ctype = CType::F32;
  int rank = 0;
  int ext[2] = {1, 1};
  size_t comps() const { return size_t(rank >= 1 ? ext[0] : 1) * size_t(rank >= 2 ? ext[1] : 1); }
  size_t elem_bytes() const { return 4; }
  size_t host_item_bytes() const { return comps() * elem_bytes(); }
  bool operator==(FieldType const &o) const {
    return ctype == o.ctype && rank == o.rank && (rank < 1 || ext[0] == o.ext[0]) && (rank < 2 || ext[1] == o.ext[1]);
  }
  bool operator!=(FieldType const &o) const { return !(*this == o); }
  bool is_real() const { return ctype == CType::F32; }
  bool is_vec3() const { return ctype == CType::F32 && rank == 1 && ext[0] == 3; }
  bool is_mat3() const { return ctype == CType::F32 && rank == 2 && ext[0] == 3 && ext[1] == 3; }
  std::string str() const;
};

FieldType parse_field_type(char const *ctype, int rank, int const *extents);

struct VaryingField {
  FieldType type;
  void *d = nullptr;   // device storage
  size_t cap = 0;      // items allocated
  uint64_t version = 0; // bumped whenever the values may have changed
  size_t device_item_bytes() const; // bytes per item of the device array (non-planar)
};

struct SmallField {
  FieldType type;
  size_t offset = 0; // byte offset in the model's arena
};

class Model;

class Group {
public:
  Group(Model *m, std::string n, std::string t) : model_(m), name(std::move(n)), type(std::move(t)) {}
  Model *model_;
  std::string name, type;
  std::set<std::string> tags;
  size_t count = 0;
  int index = 0;
  std::map<std::string, VaryingField> varying;
  std::map<std::string, SmallField> uniform;

  bool has_tag(std::string const &t) const { return tags.count(t) > 0; }
  VaryingField &add_varying(std::string const &name, FieldType const &t);
  VaryingField *find_varying(std::string const &name);
  VaryingField &get_varying(std::string const &name, FieldType const &t);
  SmallField &add_uniform(std::string const &name, FieldType const &t);
  void resize(size_t n, cudaStream_t s);
  // gather every varying field: new[i] = old[perm[i]] (device perm, uint32)
  void permute(uint32_t const *perm_d, cudaStream_t s);
  // new count n; every varying field becomes new[i] = old[src[i]], or zero
  // where src[i] == 0xFFFFFFFF (device src, uint32)
  void remap(uint32_t const *src_d, size_t n, cudaStream_t s);
};

// Scene segments of a batched model.  The items of a segmented group are
// split into consecutive ranges, one per slot (scene); the solvers then take
// every reduction and loop decision per slot, so that each scene converges
// on its own and its results do not depend on the other scenes.  Ranges are
// in slot order; an empty slot has an empty range.
struct SegGroup {
  std::vector<uint32_t> start;     // host: range of slot s is [start[s], start[s + 1])
  uint16_t *seg = nullptr;         // device: slot of each item
  uint4 *tiles = nullptr;          // device: (slot, begin, end, 0) of each tile of <= kSegTile items
  uint32_t ntiles = 0;
  uint32_t *slot_tiles = nullptr;  // device: tiles of slot s are [slot_tiles[s], slot_tiles[s + 1])
  // device: the tiles of the slots whose solver loop still iterates (the
  // first nactive[0] entries), rebuilt after each loop decision
  uint32_t *active = nullptr;
  uint32_t *nactive = nullptr; // [0] the count; [1], [2] work counters of the persistent tiled sweeps
  size_t seg_cap = 0, tile_cap = 0;
};
constexpr uint32_t kSegTile = 128; // items per reduction tile (one block)
struct Segments {
  uint32_t slots = 0;
  std::map<Group const *, SegGroup> groups;
  // per-slot device state
  double *partials = nullptr; // [3][partial_cap] tile partial sums
  size_t partial_cap = 0;
  unsigned *tickets = nullptr; // [slots] finished tiles of the running reduction
  double *scal = nullptr;      // [slots][16] solver scalars (PCG 0..7, density error 8)
  int *stat = nullptr;         // [slots][8] loop state (PCG 0..3, Jacobi 4..5)
  double *stats = nullptr;     // [slots][8] accumulated loop statistics
  int *nprde = nullptr;        // [slots] fluid items
  int *iters = nullptr;        // [slots] PCG iterations of the last solve
  uint8_t *due = nullptr;      // [slots] permute flags
  Segments() = default;
  Segments(Segments const &) = delete;
  Segments &operator=(Segments const &) = delete;
  ~Segments();
  SegGroup const *find(Group const *g) const {
    auto it = groups.find(g);
    return it == groups.end() ? nullptr : &it->second;
  }
  // set the number of slots (state of remaining slots kept, new ones zeroed)
  void set_slots(uint32_t slots, cudaStream_t s);
  void reset_slot(uint32_t slot, cudaStream_t s);
  // ranges of group g: count[s] items in slot s, consecutively in slot order
  void assign(Group const *g, std::vector<uint32_t> const &count, cudaStream_t s);
};

// Launch-shape knobs of the neighbour sweeps and the relaxed-Jacobi loop,
// set per model (by the autotuner, prtcl_gb300/tune.py, or by hand).  Every
// value gives bit-identical fields: a sweep variant changes only the
// threads per block (sweeps without a reduction), the blocks resident per SM
// (the register cap) and the neighbour-walk batch; the Jacobi value repeats
// the loop body that many times per graph iteration, the repeats past
// convergence doing nothing.  With staging, the lists of the fluid group
// also carry each entry's slot among its tile's staged items (nhood.hpp),
// and the Jacobi and PCG sweeps read their neighbours' records from shared
// memory.  The variants apply to models with one fluid and at most one
// boundary group; other layouts use variant 0 and no staging.
enum TuneKnob : int {
  kTuneDensity = 0,
  kTuneSetup,
  kTuneAccel,
  kTunePressure,
  kTuneDiag,
  kTunePcgInit,
  kTunePcgQ,
  kTuneJacobiUnroll,
  kTuneStaging,  // 1: staged lists and the staged Jacobi / PCG sweeps
  kTuneGridSort, // 1: grids of at most 128k items sorted in one launch of a thread-block cluster
  kTuneListSplit, // 1: lists of query groups of at most 64k items built by four threads per query
  kTuneKnobs
};
struct Tuning {
  int v[kTuneKnobs] = {0, 0, 0, 0, 0, 0, 0, 1, 0, 1, 1};
};
// knob names (the kernels' profiler names; "jacobi_unroll") and allowed values
char const *tune_knob_name(int k);
int tune_knob_find(std::string const &name); // -1 if unknown
bool tune_value_ok(int k, int v);
// one line per knob: "name default: value=description ..." (plain and
// batched variants differ for the reducing sweeps)
std::string tune_knob_table();

class Model {
public:
  Model();
  ~Model();
  Model(Model const &) = delete;
  Model &operator=(Model const &) = delete;

  Group &add_group(std::string const &name, std::string const &type);
  Group *find_group(std::string const &name);
  Group &group(std::string const &name);
  std::vector<Group *> groups_by_index();
  size_t group_count() const { return groups_.size(); }

  SmallField &add_global(std::string const &name, FieldType const &t);
  SmallField *find_global(std::string const &name);
  std::map<std::string, SmallField> const &globals() const { return global_; }

  // arena access
  SmallField &alloc_small(SmallField &f, FieldType const &t);
  void *small_ptr(SmallField const &f) const { return arena_d_ + f.offset; }
  void small_set(SmallField const &f, void const *host, cudaStream_t s);
  // stream-ordered set (the value travels as a kernel parameter; no host
  // synchronisation, capturable in a CUDA graph)
  void small_set_async(SmallField const &f, void const *host, cudaStream_t s);
  void small_get(SmallField const &f, void *host, cudaStream_t s);

  cudaStream_t stream() const { return stream_; }
  cudaStream_t pick(void *s) const { return s ? static_cast<cudaStream_t>(s) : stream_; }

  // bumped when groups or fields are added or a group is resized; schemes
  // loaded before such a change must be loaded again (like `model.dirty`
  // in the reference's scripts)
  uint64_t layout_version = 1;
  // device scratch shared by the procedures of this model (reductions)
  double *red_d = nullptr;       // 3 x 4096 block partial sums
  unsigned *red_count_d = nullptr; // last-block tickets
  double *scalars_d = nullptr;   // 64 FP64 solver scalars
  int *status_d = nullptr;       // 16 status words (error flags, iteration counts)
  // device-loop statistics (accumulated by the loop control kernels):
  // 0 Jacobi solves, 1 Jacobi iterations, 2 solves stopped at the cap,
  // 3 largest final aprde / nprde, 4 PCG solves, 5 PCG iterations,
  // 6 PCG solves stopped by the iteration limit
  double *stats_d = nullptr;
  void stats_reset(cudaStream_t s);
  Profiler prof;                 // optional per-kernel CUDA-event timing
  Tuning tune;                   // launch-shape knobs (all bit-identical)
  // scene segments (batched models only)
  std::unique_ptr<Segments> seg;
  // bytes of the varying fields and packed records
  size_t device_bytes() const;

  // Packed per-particle records gathered by the neighbour sweeps, rebuilt
  // only when one of their source fields changed (keyed on the fields'
  // pointers and versions):
  //   packed_xs  (x, y, z, s)       e.g. position + mass, position + volume
  //   packed_xmr (x, y, z, m / rho)
  //   packed_pr  p / (rho rho)
  float4 const *packed_xs(Group *g, VaryingField *x, VaryingField *s, char const *kind, cudaStream_t st);
  float4 const *packed_xmr(Group *g, VaryingField *x, VaryingField *m, VaryingField *rho, cudaStream_t st);
  float const *packed_pr(Group *g, VaryingField *p, VaryingField *rho, cudaStream_t st);
  // the buffer behind packed_pr, for kernels that write p and p / rho^2
  // together; pack_commit() marks it current for a key
  float *pr_buffer(Group *g, cudaStream_t st);
  void pack_commit(Group *g, std::string const &kind, std::vector<uint64_t> const &key);

private:
  struct PackEntry {
    void *d = nullptr;
    size_t cap = 0, item_bytes = 0;
    std::vector<uint64_t> key;
  };
  std::map<std::pair<Group *, std::string>, PackEntry> packs_;
  void *pack_buffer(Group *g, std::string const &kind, size_t item_bytes, std::vector<uint64_t> const &key, bool &stale,
                    cudaStream_t s);
  std::map<std::string, std::unique_ptr<Group>> groups_;
  std::map<std::string, SmallField> global_;
  char *arena_d_ = nullptr;
  size_t arena_cap_ = 0, arena_used_ = 0;
  cudaStream_t stream_ = nullptr;
  void reindex();
};

// field kernels (model.cu)
void upload_varying(VaryingField &f, size_t count, void const *host, size_t n_items, cudaStream_t s, bool sync);
// upload through a fixed static device array instead of a temporary allocation
// (noalloc.cu); synchronous, and not safe to overlap with another such call
void upload_varying_noalloc(VaryingField &f, size_t count, void const *host, size_t n_items, cudaStream_t s);
size_t noalloc_stage_bytes();
// looks up the staging array and loads its kernels on the current device
void noalloc_prepare();
void download_varying(VaryingField const &f, size_t count, void *host, size_t n_items, cudaStream_t s);
// the model in the reference's native binary archive format (archive.cu)
void save_model(Model &m, std::string const &path, cudaStream_t s);
void load_model(Model &m, std::string const &path, cudaStream_t s);
// a group as a legacy ASCII VTK file, the reference's SaveVTK format (vtk.cu)
void save_vtk(Group &g, std::string const &path, cudaStream_t s);
// items [offset, offset + n) of a field, in the host layout (stream-ordered;
// the download synchronises)
void upload_varying_range(VaryingField &f, size_t offset, void const *host, size_t n, cudaStream_t s);
void download_varying_range(VaryingField const &f, size_t offset, void *host, size_t n, cudaStream_t s);

} // namespace prtcl_gpu
