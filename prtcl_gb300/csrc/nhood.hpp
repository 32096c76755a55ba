// Device uniform-grid neighbourhood: the GB300 replacement for prtcl's
// grouped_uniform_grid (util/grouped_uniform_grid.hpp) behind the
// Neighborhood interface (util/neighborhood.hpp:23-42).
//
// Update():
//   1. cell of every item of every neighbour-capable group:
//      gi = (int32) floor((double) x / radius)            (:621-632)
//   2. a 64-bit Z-order key per item.  The reference compares cells with an
//      XOR-MSB test on u = (uint32) gi + INT32_MAX (util/morton_order.hpp:
//      40-82); that order equals the order of the 96-bit interleave of
//      (u0, u1, u2) with dimension 0 the most significant of each bit triple.
//      Bit positions that carry no information for the current item set are
//      deleted before interleaving: bits that are constant, and bits that
//      are always equal (or always unequal) to bit 31 (with the INT32_MAX bias
//      every cell near the origin has bits 30..k equal to NOT bit 31).
//      Deleting such positions keeps both the monotonicity of each axis and
//      the order of most-significant differing bits across axes, so the
//      compressed key orders cells exactly like the reference.  At most 21
//      informative bits per axis are supported (63-bit keys).
//   3. a stable LSD radix sort of (key, handle) pairs, 8-bit digits, starting
//      from group-major identity order: cells in the reference's Morton
//      order; within a cell (group, raw index) order.  The reference's
//      parallel sort is unstable, so its within-cell order is unspecified;
//      cell membership and cell order are exact.
//   4. cell boundaries, cell ids by prefix scan, cell ranges, cell keys and
//      grid indices, and raw -> sorted.
//   5. the 26-cell adjacency: slot k < 13 holds the cell at +offset[k],
//      slot 25-k the cell at -offset[k] (:52-68, :312-337); found by binary
//      search over the sorted cell keys.
// Neighbour lists (built lazily per query group, reused by every procedure
// until positions change or the grid is updated): for each query item the
// own cell and adjacency slots 0..25 in order, each cell's items in sorted
// order, kept when (double)(float)|x_i - x_j|^2 < r^2 (:407-422).  One ELL
// array per neighbour group (idx[slot * n + i]) so that a procedure walks
// its fluid and boundary neighbours without branching on the group.
#pragma once

#include "model.hpp"

#include <map>
#include <vector>

namespace prtcl_gpu {

// Device view of the neighbour lists of one query group, one set per
// neighbour group g.  In 96-byte chunks of 16 entries: chunk c of item i
// holds its entries 16c..16c+15 as
//   16 x uint16  j - base   (32 bytes)
//   16 x float   the pair's kernel-gradient factor (64 bytes)
// so a chunk is exactly three 32-byte sectors and every fetched sector is
// used once (offsets are signed 16-bit: j = base + offset).  Chunk-major:
// chunk c of item i sits at chunks[(c * n + i) * 96], so that the threads
// of a warp, walking consecutive items, read their chunk c from one
// contiguous 3 KB span.  Also per item:
//   cb[g][i]    (count | kWide if "wide", base = the first neighbour's index)
//   idx32[g]    j as 32-bit indices at [i * cap + k], written and read for
//               "wide" items only (neighbours spanning >= 65536 indices)
// The factors are present when the lists were built with a smoothing scale
// (hcache, device); kernels use them only while hcache equals the current
// smoothing scale and evaluate the gradient in full otherwise.
constexpr uint32_t kChunk = 16;
constexpr uint32_t kChunkBytes = kChunk * 2 + kChunk * 4;
// Staged lists (built on request for a query group in cell order): the
// query items form tiles of kStageTile consecutive items (the list build's
// blocks, and the staged sweeps' blocks).  The cells adjacent to a tile's
// cells (own cell included) are its staged cells; their sorted items, cell
// after cell in the tile's table order, are the tile's staged items, at most
// kStageCap.  Besides the offsets and factors, each entry then has its
// neighbour's position among the tile's staged items (slot, 16 bits),
// chunk-major like the offsets (chunk c of item i at (c * n + i), 16 slots
// of 2 bytes), so that a sweep that copies a tile's staged items to shared
// memory reads its gathers from there.  tile_info[t] = (staged cells, staged
// items), the items 0xFFFFFFFF for a tile that did not fit (no slots; the
// sweep takes the offsets); tile_cells[t * kStageCells + u] = (first sorted
// index of the cell, its first staged slot).
constexpr uint32_t kStageTile = 128;
constexpr uint32_t kStageCap = 1536;
constexpr uint32_t kStageCells = 256;
constexpr uint32_t kStageHash = 512;
constexpr uint32_t kNoStage = 0xFFFFFFFFu;
struct NbrView {
  unsigned char const *chunks[kMaxGroups];
  uint32_t const *idx32[kMaxGroups];
  uint2 const *cb[kMaxGroups];
  uint32_t cap[kMaxGroups]; // a multiple of kChunk
  uint32_t n;               // query items
  float const *hcache;      // NaN when no factors were computed
  // staged lists (nullptr when not built staged)
  uint16_t const *slots[kMaxGroups];
  uint2 const *tile_info;
  uint2 const *tile_cells;
};

constexpr uint32_t kWide = 0x80000000u;

// host decode of entry k of item i, with `chunks` a host copy of the
// chunk-major array of n items: the 16-bit entries are signed offsets from
// the row's base (its first neighbour)
inline uint32_t nbr_host_decode(uint2 cb, unsigned char const *chunks, size_t n, size_t i, uint32_t const *idx32row,
                                uint32_t k) {
  if (cb.x & kWide) return idx32row[k];
  unsigned char const *p = chunks + (size_t(k / kChunk) * n + i) * kChunkBytes + (k % kChunk) * 2;
  int16_t d = int16_t(uint16_t(p[0] | (p[1] << 8)));
  return cb.y + uint32_t(int32_t(d));
}

constexpr int kMaxListGroups = 8; // groups a neighbour-list build supports

constexpr int kKeyRuns = 4; // runs of kept bits gathered without a bit loop

struct KeyInfo {
  uint32_t keep = 0;   // informative bit positions of u
  uint32_t rel_eq = 0; // deleted low positions always equal to bit 31
  uint32_t rel_ne = 0; // deleted low positions always unequal to bit 31
  uint32_t b31_const = 0; // value of bit 31 if deleted (0 or 0x80000000)
  int bits = 0;        // informative bits per axis
  // `keep` as runs of consecutive bits, when it has at most kKeyRuns of
  // them (nruns = 0 otherwise): the gather of run r is
  // (u & run_mask[r]) >> run_shift[r]
  int nruns = 0;
  uint32_t run_mask[kKeyRuns] = {};
  uint32_t run_shift[kKeyRuns] = {};
};

// split `keep` into runs of consecutive set bits (at most kKeyRuns)
inline void key_runs(KeyInfo &k) {
  k.nruns = 0;
  uint32_t m = k.keep;
  int out = 0; // output position of the next run
  while (m) {
    if (k.nruns == kKeyRuns) {
      k.nruns = 0;
      return;
    }
    int lo = __builtin_ctz(m);
    uint32_t low = m >> lo;
    int len = (low == 0xFFFFFFFFu) ? 32 : __builtin_ctz(~low);
    uint32_t rm = (len == 32 ? 0xFFFFFFFFu : ((1u << len) - 1u)) << lo;
    k.run_mask[k.nruns] = rm;
    k.run_shift[k.nruns] = uint32_t(lo - out);
    ++k.nruns;
    out += len;
    m &= ~rm;
  }
}

struct GridView {
  uint32_t const *sorted;   // sorted -> handle (group << 28 | index)
  int32_t const *r2s;       // raw -> sorted, at goff[group] + index
  int32_t const *s2c;       // sorted -> cell
  int32_t const *cell_start; // cell -> first sorted (C + 1 entries)
  uint64_t const *cell_key; // cell -> compressed key
  int32_t const *cell_adj;  // cell -> 26 adjacent cells (-1 none)
  int4 const *cell_gi;      // cell -> grid index
  int const *ncells;        // number of cells (device)
  uint32_t goff[kMaxGroups + 1];
  int in_grid[kMaxGroups];
  KeyInfo key;
  // batched models: per group the segment (scene) of each item, or nullptr
  // (segment 0); the segment sits above the Z-order bits of the cell key,
  // at bit seg_shift, so that cells of different segments never meet
  uint16_t const *seg[kMaxGroups];
  int seg_shift;
  double radius, r2;
  float rinv;  // 1 / radius rounded to f32 (fast path of the cell index)
  float r2lt;  // d2 < r2lt  <=>  (double) d2 < r2, for every float d2
};

class Nhood {
public:
  Nhood();
  ~Nhood();
  Nhood(Nhood const &) = delete;
  Nhood &operator=(Nhood const &) = delete;

  void set_radius(double r) { radius_ = r; }
  double radius() const { return radius_; }
  void load(Model &m);
  void update(cudaStream_t s);
  void permute(Model &m, cudaStream_t s);
  // Permute restricted to the segments whose flag is set in due_d (device,
  // one byte per segment); the items of other segments keep their order.
  // Only for segmented groups: segments occupy consecutive index ranges and
  // the segment is the most significant part of the cell key, so the
  // permutation never moves an item out of its segment's range.
  void permute_segments(Model &m, uint8_t const *due_d, cudaStream_t s);
  // Split the items of every group into segments (scenes of a batched
  // model): seg[g] gives the segment of each item of group g (device, may
  // be nullptr for segment 0), `count` segments in all (0: unsegmented).
  // Invalidates the grid.
  void set_segments(std::vector<uint16_t const *> const &seg, uint32_t count);
  bool loaded() const { return model_ != nullptr; }
  Model *model() const { return model_; }

  // neighbour lists of query group q (rebuilt when stale); with `h` (the
  // smoothing scale on the device) they also hold each pair's kernel
  // gradient factor
  NbrView const &lists(int q, cudaStream_t s, float const *h = nullptr, bool stage = false);

  // introspection (tests): sizes and host copies of the grid
  size_t sorted_count() const { return N_; }
  size_t cell_count(cudaStream_t s);
  void copy_grid(uint32_t *sorted, int32_t *cell_gi, int32_t *cell_range, int32_t *cell_adj, cudaStream_t s);
  // neighbours of one item, per group, like Neighborhood::CopyNeighbors
  size_t copy_neighbors(int g, size_t i, int64_t *counts, int64_t *out, size_t cap, cudaStream_t s);
  // total neighbour count of the lists of query group q (synchronises)
  uint64_t pair_count(int q, cudaStream_t s);
  // CSR copy of the lists of query group q to neighbour group ng
  void copy_lists(int q, int ng, int64_t *offsets, uint32_t *idx, size_t cap, cudaStream_t s);
  // tiles of query group q's last built lists whose staged records fit, and
  // all tiles (0, 0 when they were not built staged; synchronises)
  size_t staged_tiles(int q, size_t &tiles, cudaStream_t s);

  GridView view() const;
  // sorted positions with their handles in w (current after the lists of a
  // group have been built for the present positions)
  float4 const *sorted_positions() const { return xsorted_; }
  // bytes of the grid arrays and the neighbour lists
  size_t device_bytes() const;
  uint64_t epoch() const { return epoch_; }
  // informative-bit overflow and other errors raise; lists growth is handled
  int list_rebuilds = 0;

private:
  struct GG {
    Group *g = nullptr;
    VaryingField *pos = nullptr;
    bool can_be_neighbor = false;
  };
  struct Lists {
    size_t n = 0;
    uint32_t cap[kMaxGroups] = {};
    uint32_t *idx32[kMaxGroups] = {};
    unsigned char *chunks[kMaxGroups] = {};
    uint16_t *slots[kMaxGroups] = {};   // staged lists only
    uint2 *tile_info = nullptr, *tile_cells = nullptr;
    size_t tile_cap = 0;
    bool staged = false;
    uint2 *cb = nullptr; // [G][n]
    float *hcache = nullptr;
    bool has_gf = false;
    uint64_t epoch = 0;
    std::vector<uint64_t> pos_versions;
    NbrView view{};
  };
  void ensure_grid_capacity(size_t n);
  void build_lists(int q, Lists &L, cudaStream_t s, float const *h, bool stage);
  // Confirm the key layout an update took from the previous one (one
  // synchronisation); on a mismatch, update again with a layout read back
  // first.  Called before the grid is read on the host or permutes fields;
  // the list build confirms it at its own synchronisation instead.
  void settle(cudaStream_t s);
  bool lists_fresh(Lists const &L) const;
  std::vector<uint64_t> pos_versions() const;
  void free_lists(Lists &L);

  double radius_ = 1.0;
  Model *model_ = nullptr;
  std::vector<GG> gg_;
  size_t N_ = 0, cap_ = 0;
  uint32_t goff_[kMaxGroups + 1] = {};
  int in_grid_[kMaxGroups] = {};
  KeyInfo key_{};
  // The cell-key layout is a function of four bit statistics of all items'
  // grid indices (k_cells_u).  An update reuses the last layout without
  // reading the statistics back (key_known_), and flags it for the check
  // (key_check_) at the next synchronisation; in a simulation the layout
  // changes only when the particles' grid indices gain or lose bit patterns.
  bool key_known_ = false, key_check_ = false;
  // item count of each group when it was last permuted into cell order (the
  // list build walks a group that was not in grid order instead)
  size_t permuted_count_[kMaxGroups] = {};
  uint32_t *order_ = nullptr; // group items in grid order (list build)
  uint64_t *hkeys_ = nullptr;  // cell-key hash table (adjacency lookups)
  int32_t *hvals_ = nullptr;
  size_t hash_cap_ = 0;
  size_t order_cap_ = 0;
  std::vector<uint16_t const *> seg_;
  uint32_t seg_count_ = 0;
  int seg_bits_ = 0;
  uint64_t epoch_ = 0;
  bool has_grid_ = false;

  // device arrays (capacity cap_)
  uint64_t *keys_a_ = nullptr, *keys_b_ = nullptr;
  uint32_t *vals_a_ = nullptr, *vals_b_ = nullptr;
  uint32_t *ukeys_ = nullptr; // 4 words per item (u0, u1, u2, pad)
  uint32_t *flags_ = nullptr, *scan_ = nullptr;
  int32_t *r2s_ = nullptr, *s2c_ = nullptr, *cell_start_ = nullptr, *cell_adj_ = nullptr;
  uint64_t *cell_key_ = nullptr;
  int4 *cell_gi_ = nullptr;
  float4 *xsorted_ = nullptr;
  uint32_t *hist_ = nullptr;
  size_t hist_cap_ = 0;
  uint32_t *block_sums_ = nullptr;
  size_t block_sums_cap_ = 0;
  uint32_t *stats_d_ = nullptr; // bit statistics / counters (16 words)
  int *ncells_d_ = nullptr;
  uint32_t *stats_h_ = nullptr; // pinned
  uint64_t const *sorted_keys_ = nullptr;
  uint32_t const *sorted_vals_ = nullptr;
  std::map<int, Lists> lists_;
};

} // namespace prtcl_gpu
