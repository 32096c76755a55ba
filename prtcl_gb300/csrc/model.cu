// Device data model: groups, varying / uniform / global fields, upload,
// download and the per-group permutation gather (data/varying_manager.hpp:
// 86-101 applies new[i] = old[perm[i]] to every varying field of a group).
#include "model.hpp"

#include <algorithm>
#include <cstring>
#include <type_traits>

namespace prtcl_gpu {

std::string FieldType::str() const {
  std::string s = ctype == CType::F32 ? "real" : "integer";
  for (int r = 0; r < rank; ++r) s += "[" + std::to_string(ext[r]) + "]";
  return s;
}

FieldType parse_field_type(char const *ctype, int rank, int const *extents) {
  FieldType t;
  std::string c = ctype ? ctype : "";
  if (c == "f32" || c == "real" || c == "float32") t.ctype = CType::F32;
  else if (c == "i32" || c == "integer" || c == "int32") t.ctype = CType::I32;
  else throw Error("unsupported component type '" + c + "' (device fields are f32 or i32)");
  if (rank < 0 || rank > 2) throw Error("unsupported field rank " + std::to_string(rank));
  t.rank = rank;
  for (int r = 0; r < rank; ++r) {
    if (!extents || extents[r] <= 0) throw Error("invalid field extent");
    t.ext[r] = extents[r];
  }
  return t;
}

size_t VaryingField::device_item_bytes() const {
  if (type.is_vec3()) return 16;
  return type.host_item_bytes();
}

// ---------------------------------------------------------------------------
// kernels
// ---------------------------------------------------------------------------

__global__ void k_expand_vec3(float const *__restrict__ src, float4 *__restrict__ dst, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) dst[i] = make_float4(src[3 * i], src[3 * i + 1], src[3 * i + 2], 0.0f);
}
__global__ void k_pack_vec3(float4 const *__restrict__ src, float *__restrict__ dst, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    float4 v = src[i];
    dst[3 * i] = v.x;
    dst[3 * i + 1] = v.y;
    dst[3 * i + 2] = v.z;
  }
}
// host layout: 9 floats per item (column-major); device: plane k at k*cap
__global__ void k_to_planar9(float const *__restrict__ src, float *__restrict__ dst, size_t n, size_t cap) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n)
    for (int k = 0; k < 9; ++k) dst[k * cap + i] = src[9 * i + k];
}
__global__ void k_from_planar9(float const *__restrict__ src, float *__restrict__ dst, size_t n, size_t cap) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n)
    for (int k = 0; k < 9; ++k) dst[9 * i + k] = src[k * cap + i];
}
template <class V>
__global__ void k_gather(V const *__restrict__ src, V *__restrict__ dst, uint32_t const *__restrict__ perm, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) dst[i] = src[perm[i]];
}
__global__ void k_gather_planar9(float const *__restrict__ src, float *__restrict__ dst, uint32_t const *__restrict__ perm,
                                 size_t n, size_t scap, size_t dcap) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    uint32_t j = perm[i];
    for (int k = 0; k < 9; ++k) dst[k * dcap + i] = src[k * scap + j];
  }
}
// generic item gather in 4-byte words
__global__ void k_gather_words(uint32_t const *__restrict__ src, uint32_t *__restrict__ dst,
                               uint32_t const *__restrict__ perm, size_t n, int words) {
  size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  size_t i = t / words;
  int w = int(t % words);
  if (i < n) dst[i * words + w] = src[size_t(perm[i]) * words + w];
}

// remap gathers: src index 0xFFFFFFFF gives zero
constexpr uint32_t kNoSrc = 0xFFFFFFFFu;
template <class V>
__global__ void k_remap(V const *__restrict__ src, V *__restrict__ dst, uint32_t const *__restrict__ map, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    uint32_t j = map[i];
    if (j != kNoSrc) dst[i] = src[j];
  }
}
__global__ void k_remap_planar9(float const *__restrict__ src, float *__restrict__ dst, uint32_t const *__restrict__ map,
                                size_t n, size_t scap, size_t dcap) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    uint32_t j = map[i];
    if (j != kNoSrc)
      for (int k = 0; k < 9; ++k) dst[k * dcap + i] = src[k * scap + j];
  }
}
__global__ void k_remap_words(uint32_t const *__restrict__ src, uint32_t *__restrict__ dst,
                              uint32_t const *__restrict__ map, size_t n, int words) {
  size_t t = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  size_t i = t / words;
  int w = int(t % words);
  if (i < n && map[i] != kNoSrc) dst[i * words + w] = src[size_t(map[i]) * words + w];
}
// slot of each item of a segmented group, from the tiles
__global__ void k_fill_seg(uint4 const *tiles, uint32_t ntiles, uint16_t *seg) {
  uint32_t t = blockIdx.x;
  if (t >= ntiles) return;
  uint4 T = tiles[t];
  uint32_t i = T.y + threadIdx.x;
  if (i < T.z) seg[i] = uint16_t(T.x);
}

// ---------------------------------------------------------------------------
// storage helpers
// ---------------------------------------------------------------------------

static void *alloc_field(FieldType const &t, size_t cap, cudaStream_t s) {
  size_t bytes = t.is_vec3() ? cap * 16 : cap * t.host_item_bytes();
  if (bytes == 0) return nullptr;
  void *p = nullptr;
  PG_CUDA(cudaMallocAsync(&p, bytes, s));
  PG_CUDA(cudaMemsetAsync(p, 0, bytes, s));
  return p;
}

static void copy_items(VaryingField const &src, void *dst, size_t dst_cap, size_t n, cudaStream_t s) {
  if (n == 0) return;
  if (src.type.is_mat3()) {
    for (int k = 0; k < 9; ++k)
      PG_CUDA(cudaMemcpyAsync(static_cast<float *>(dst) + k * dst_cap, static_cast<float *>(src.d) + k * src.cap,
                              n * 4, cudaMemcpyDeviceToDevice, s));
  } else {
    PG_CUDA(cudaMemcpyAsync(dst, src.d, n * src.device_item_bytes(), cudaMemcpyDeviceToDevice, s));
  }
}

void upload_varying(VaryingField &f, size_t count, void const *host, size_t n_items, cudaStream_t s, bool sync) {
  if (n_items != count)
    throw Error("upload: item count " + std::to_string(n_items) + " != group count " + std::to_string(count));
  f.version++;
  if (count == 0) return;
  size_t hbytes = count * f.type.host_item_bytes();
  if (!f.type.is_vec3() && !f.type.is_mat3()) {
    PG_CUDA(cudaMemcpyAsync(f.d, host, hbytes, cudaMemcpyHostToDevice, s));
  } else {
    void *stage = nullptr;
    PG_CUDA(cudaMallocAsync(&stage, hbytes, s));
    PG_CUDA(cudaMemcpyAsync(stage, host, hbytes, cudaMemcpyHostToDevice, s));
    if (f.type.is_vec3())
      k_expand_vec3<<<div_up(count, 256), 256, 0, s>>>(static_cast<float *>(stage), static_cast<float4 *>(f.d), count);
    else
      k_to_planar9<<<div_up(count, 256), 256, 0, s>>>(static_cast<float *>(stage), static_cast<float *>(f.d), count, f.cap);
    count_launch();
    PG_LAUNCH_CHECK();
    PG_CUDA(cudaFreeAsync(stage, s));
  }
  if (sync) PG_CUDA(cudaStreamSynchronize(s));
}

void upload_varying_range(VaryingField &f, size_t offset, void const *host, size_t n, cudaStream_t s) {
  if (offset + n > f.cap) throw Error("upload: range beyond the field");
  f.version++;
  if (n == 0) return;
  size_t hbytes = n * f.type.host_item_bytes();
  if (!f.type.is_vec3() && !f.type.is_mat3()) {
    PG_CUDA(cudaMemcpyAsync(static_cast<char *>(f.d) + offset * f.type.host_item_bytes(), host, hbytes,
                            cudaMemcpyHostToDevice, s));
    return;
  }
  void *stage = nullptr;
  PG_CUDA(cudaMallocAsync(&stage, hbytes, s));
  PG_CUDA(cudaMemcpyAsync(stage, host, hbytes, cudaMemcpyHostToDevice, s));
  if (f.type.is_vec3())
    k_expand_vec3<<<div_up(n, 256), 256, 0, s>>>(static_cast<float *>(stage), static_cast<float4 *>(f.d) + offset, n);
  else
    k_to_planar9<<<div_up(n, 256), 256, 0, s>>>(static_cast<float *>(stage), static_cast<float *>(f.d) + offset, n,
                                                 f.cap);
  count_launch();
  PG_LAUNCH_CHECK();
  PG_CUDA(cudaFreeAsync(stage, s));
}

void download_varying_range(VaryingField const &f, size_t offset, void *host, size_t n, cudaStream_t s) {
  if (offset + n > f.cap) throw Error("download: range beyond the field");
  if (n == 0) return;
  size_t hbytes = n * f.type.host_item_bytes();
  if (!f.type.is_vec3() && !f.type.is_mat3()) {
    PG_CUDA(cudaMemcpyAsync(host, static_cast<char const *>(f.d) + offset * f.type.host_item_bytes(), hbytes,
                            cudaMemcpyDeviceToHost, s));
  } else {
    void *stage = nullptr;
    PG_CUDA(cudaMallocAsync(&stage, hbytes, s));
    if (f.type.is_vec3())
      k_pack_vec3<<<div_up(n, 256), 256, 0, s>>>(static_cast<float4 const *>(f.d) + offset, static_cast<float *>(stage),
                                                 n);
    else
      k_from_planar9<<<div_up(n, 256), 256, 0, s>>>(static_cast<float const *>(f.d) + offset,
                                                    static_cast<float *>(stage), n, f.cap);
    count_launch();
    PG_LAUNCH_CHECK();
    PG_CUDA(cudaMemcpyAsync(host, stage, hbytes, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaFreeAsync(stage, s));
  }
  PG_CUDA(cudaStreamSynchronize(s));
}

void download_varying(VaryingField const &f, size_t count, void *host, size_t n_items, cudaStream_t s) {
  if (n_items != count)
    throw Error("download: item count " + std::to_string(n_items) + " != group count " + std::to_string(count));
  if (count == 0) return;
  size_t hbytes = count * f.type.host_item_bytes();
  if (!f.type.is_vec3() && !f.type.is_mat3()) {
    PG_CUDA(cudaMemcpyAsync(host, f.d, hbytes, cudaMemcpyDeviceToHost, s));
  } else {
    void *stage = nullptr;
    PG_CUDA(cudaMallocAsync(&stage, hbytes, s));
    if (f.type.is_vec3())
      k_pack_vec3<<<div_up(count, 256), 256, 0, s>>>(static_cast<float4 const *>(f.d), static_cast<float *>(stage), count);
    else
      k_from_planar9<<<div_up(count, 256), 256, 0, s>>>(static_cast<float const *>(f.d), static_cast<float *>(stage), count, f.cap);
    count_launch();
    PG_LAUNCH_CHECK();
    PG_CUDA(cudaMemcpyAsync(host, stage, hbytes, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaFreeAsync(stage, s));
  }
  PG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// Group
// ---------------------------------------------------------------------------

VaryingField &Group::add_varying(std::string const &n, FieldType const &t) {
  auto it = varying.find(n);
  if (it != varying.end()) {
    if (it->second.type != t) throw Error("field of different type already exists: " + name + "." + n);
    return it->second;
  }
  VaryingField f;
  f.type = t;
  f.cap = count;
  f.d = alloc_field(t, count, model_->stream());
  model_->layout_version++;
  return varying.emplace(n, f).first->second;
}

VaryingField *Group::find_varying(std::string const &n) {
  auto it = varying.find(n);
  return it == varying.end() ? nullptr : &it->second;
}

VaryingField &Group::get_varying(std::string const &n, FieldType const &t) {
  auto *f = find_varying(n);
  if (!f) throw Error("field does not exist: " + name + "." + n);
  if (f->type != t) throw Error("field " + name + "." + n + " is " + f->type.str() + ", expected " + t.str());
  return *f;
}

SmallField &Group::add_uniform(std::string const &n, FieldType const &t) {
  auto it = uniform.find(n);
  if (it != uniform.end()) {
    if (it->second.type != t) throw Error("uniform field of different type already exists: " + name + "." + n);
    return it->second;
  }
  SmallField &f = uniform[n];
  return model_->alloc_small(f, t);
}

void Group::resize(size_t n, cudaStream_t s) {
  if (n >= (size_t(1) << 28)) throw Error("group '" + name + "' too large: at most 2^28 - 1 items");
  if (n == count) return;
  for (auto &kv : varying) {
    VaryingField &f = kv.second;
    void *nd = alloc_field(f.type, n, s);
    copy_items(f, nd, n, std::min(n, count), s);
    if (f.d) PG_CUDA(cudaFreeAsync(f.d, s));
    f.d = nd;
    f.cap = n;
    f.version++;
  }
  count = n;
  model_->layout_version++;
}

// Gathers into scratch and copies back, so that field pointers stay stable
// (captured CUDA graphs and bound kernels keep working after a permute).
void Group::permute(uint32_t const *perm, cudaStream_t s) {
  size_t n = count;
  if (n == 0) return;
  for (auto &kv : varying) {
    VaryingField &f = kv.second;
    void *nd = alloc_field(f.type, f.cap, s);
    unsigned b = 256;
    if (f.type.is_vec3()) {
      k_gather<float4><<<div_up(n, b), b, 0, s>>>(static_cast<float4 const *>(f.d), static_cast<float4 *>(nd), perm, n); count_launch();
    } else if (f.type.is_mat3()) {
      k_gather_planar9<<<div_up(n, b), b, 0, s>>>(static_cast<float const *>(f.d), static_cast<float *>(nd), perm, n,
                                                  f.cap, f.cap); count_launch();
    } else if (f.type.host_item_bytes() == 4) {
      k_gather<uint32_t><<<div_up(n, b), b, 0, s>>>(static_cast<uint32_t const *>(f.d), static_cast<uint32_t *>(nd), perm, n); count_launch();
    } else {
      int words = int(f.type.host_item_bytes() / 4);
      k_gather_words<<<div_up(n * words, b), b, 0, s>>>(static_cast<uint32_t const *>(f.d), static_cast<uint32_t *>(nd),
                                                        perm, n, words); count_launch();
    }
    PG_LAUNCH_CHECK();
    size_t bytes = f.type.is_vec3() ? f.cap * 16 : f.cap * f.type.host_item_bytes();
    PG_CUDA(cudaMemcpyAsync(f.d, nd, bytes, cudaMemcpyDeviceToDevice, s));
    PG_CUDA(cudaFreeAsync(nd, s));
    f.version++;
  }
}

void Group::remap(uint32_t const *map, size_t n, cudaStream_t s) {
  if (n >= (size_t(1) << 28)) throw Error("group '" + name + "' too large: at most 2^28 - 1 items");
  for (auto &kv : varying) {
    VaryingField &f = kv.second;
    void *nd = alloc_field(f.type, n, s); // zeroed
    unsigned b = 256;
    if (n) {
      if (f.type.is_vec3()) {
        k_remap<float4><<<div_up(n, b), b, 0, s>>>(static_cast<float4 const *>(f.d), static_cast<float4 *>(nd), map, n);
      } else if (f.type.is_mat3()) {
        k_remap_planar9<<<div_up(n, b), b, 0, s>>>(static_cast<float const *>(f.d), static_cast<float *>(nd), map, n,
                                                   f.cap, n);
      } else if (f.type.host_item_bytes() == 4) {
        k_remap<uint32_t><<<div_up(n, b), b, 0, s>>>(static_cast<uint32_t const *>(f.d), static_cast<uint32_t *>(nd),
                                                      map, n);
      } else {
        int words = int(f.type.host_item_bytes() / 4);
        k_remap_words<<<div_up(n * words, b), b, 0, s>>>(static_cast<uint32_t const *>(f.d),
                                                          static_cast<uint32_t *>(nd), map, n, words);
      }
      count_launch();
      PG_LAUNCH_CHECK();
    }
    if (f.d) PG_CUDA(cudaFreeAsync(f.d, s));
    f.d = nd;
    f.cap = n;
    f.version++;
  }
  count = n;
  model_->layout_version++;
}

// ---------------------------------------------------------------------------
// segments
// ---------------------------------------------------------------------------

Segments::~Segments() {
  for (auto &kv : groups) {
    if (kv.second.seg) cudaFree(kv.second.seg);
    if (kv.second.tiles) cudaFree(kv.second.tiles);
    if (kv.second.slot_tiles) cudaFree(kv.second.slot_tiles);
    if (kv.second.active) cudaFree(kv.second.active);
    if (kv.second.nactive) cudaFree(kv.second.nactive);
  }
  for (void *p : {(void *)partials, (void *)tickets, (void *)scal, (void *)stat, (void *)stats, (void *)nprde,
                  (void *)iters, (void *)due})
    if (p) cudaFree(p);
}

// Slot state is kept across a change of the slot count (slots that stay keep
// their statistics); new slots start zeroed.
void Segments::set_slots(uint32_t n, cudaStream_t s) {
  if (n > 65536) throw Error("at most 65536 segments");
  if (n == slots && tickets) return;
  size_t m = std::max<uint32_t>(n, 1), keep = std::min(n, slots);
  auto grow = [&](auto *&p, size_t per) {
    using T = std::remove_reference_t<decltype(*p)>;
    T *q = nullptr;
    PG_CUDA(cudaMalloc(&q, m * per * sizeof(T)));
    PG_CUDA(cudaMemsetAsync(q, 0, m * per * sizeof(T), s));
    if (p && keep) PG_CUDA(cudaMemcpyAsync(q, p, keep * per * sizeof(T), cudaMemcpyDeviceToDevice, s));
    if (p) {
      PG_CUDA(cudaStreamSynchronize(s));
      PG_CUDA(cudaFree(p));
    }
    p = q;
  };
  grow(tickets, 1);
  grow(scal, 16);
  grow(stat, 8);
  grow(stats, 8);
  grow(nprde, 1);
  grow(iters, 1);
  grow(due, 1);
  slots = n;
}

// zero the state of one slot (a scene that takes the slot over)
void Segments::reset_slot(uint32_t k, cudaStream_t s) {
  if (k >= slots) throw Error("segments: slot out of range");
  PG_CUDA(cudaMemsetAsync(tickets + k, 0, sizeof(unsigned), s));
  PG_CUDA(cudaMemsetAsync(scal + size_t(k) * 16, 0, 16 * sizeof(double), s));
  PG_CUDA(cudaMemsetAsync(stat + size_t(k) * 8, 0, 8 * sizeof(int), s));
  PG_CUDA(cudaMemsetAsync(stats + size_t(k) * 8, 0, 8 * sizeof(double), s));
  PG_CUDA(cudaMemsetAsync(iters + k, 0, sizeof(int), s));
  PG_CUDA(cudaMemsetAsync(due + k, 0, 1, s));
}

void Segments::assign(Group const *g, std::vector<uint32_t> const &count, cudaStream_t s) {
  if (count.size() != slots) throw Error("segments: one count per slot expected");
  SegGroup &G = groups[g];
  G.start.assign(slots + 1, 0);
  std::vector<uint4> tiles;
  std::vector<uint32_t> slot_tiles(slots + 1, 0);
  for (uint32_t k = 0; k < slots; ++k) {
    G.start[k + 1] = G.start[k] + count[k];
    slot_tiles[k] = uint32_t(tiles.size());
    for (uint32_t b = G.start[k]; b < G.start[k + 1]; b += kSegTile)
      tiles.push_back(make_uint4(k, b, std::min(b + kSegTile, G.start[k + 1]), 0u));
  }
  slot_tiles[slots] = uint32_t(tiles.size());
  size_t n = G.start[slots];
  if (n != g->count) throw Error("segments of group '" + g->name + "' do not cover its items");
  if (n > G.seg_cap) {
    if (G.seg) PG_CUDA(cudaFree(G.seg));
    G.seg_cap = std::max<size_t>(n + n / 8, 1024);
    PG_CUDA(cudaMalloc(&G.seg, G.seg_cap * sizeof(uint16_t)));
  }
  if (tiles.size() + 1 > G.tile_cap || slots + 1 > G.tile_cap) {
    if (G.tiles) PG_CUDA(cudaFree(G.tiles));
    if (G.slot_tiles) PG_CUDA(cudaFree(G.slot_tiles));
    if (G.active) PG_CUDA(cudaFree(G.active));
    G.tile_cap = std::max<size_t>(std::max(tiles.size(), size_t(slots)) + 1024, 4096);
    PG_CUDA(cudaMalloc(&G.tiles, G.tile_cap * sizeof(uint4)));
    PG_CUDA(cudaMalloc(&G.slot_tiles, G.tile_cap * sizeof(uint32_t)));
    PG_CUDA(cudaMalloc(&G.active, G.tile_cap * sizeof(uint32_t)));
    // [0] active tiles, [1] and [2] the work counters of the persistent
    // tiled Jacobi sweeps
    if (!G.nactive) {
      PG_CUDA(cudaMalloc(&G.nactive, 4 * sizeof(uint32_t)));
      PG_CUDA(cudaMemsetAsync(G.nactive, 0, 4 * sizeof(uint32_t), s));
    }
  }
  G.ntiles = uint32_t(tiles.size());
  if (!tiles.empty())
    PG_CUDA(cudaMemcpyAsync(G.tiles, tiles.data(), tiles.size() * sizeof(uint4), cudaMemcpyHostToDevice, s));
  PG_CUDA(cudaMemcpyAsync(G.slot_tiles, slot_tiles.data(), slot_tiles.size() * sizeof(uint32_t),
                          cudaMemcpyHostToDevice, s));
  if (G.ntiles) {
    k_fill_seg<<<G.ntiles, kSegTile, 0, s>>>(G.tiles, G.ntiles, G.seg);
    count_launch();
    PG_LAUNCH_CHECK();
  }
  if (G.ntiles > partial_cap) {
    if (partials) PG_CUDA(cudaFree(partials));
    partial_cap = size_t(G.ntiles) + G.ntiles / 4 + 1024;
    PG_CUDA(cudaMalloc(&partials, 3 * partial_cap * sizeof(double)));
  }
  // the host copies above read pageable vectors: finish before they go away
  PG_CUDA(cudaStreamSynchronize(s));
}

// ---------------------------------------------------------------------------
// packed neighbour records
// ---------------------------------------------------------------------------

__global__ void k_pack_xs(float4 const *__restrict__ x, float const *__restrict__ sc, float4 *__restrict__ out, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    float4 v = x[i];
    v.w = sc[i];
    out[i] = v;
  }
}
// x and m / rho (the ratio the viscosity sums use, computed as m_j / rho_j)
__global__ void k_pack_xmr(float4 const *__restrict__ x, float const *__restrict__ m, float const *__restrict__ rho,
                           float4 *__restrict__ out, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    float4 v = x[i];
    v.w = m[i] / rho[i];
    out[i] = v;
  }
}
// p / (rho rho), the pressure term of the pressure acceleration
__global__ void k_pack_pr(float const *__restrict__ p, float const *__restrict__ rho, float *__restrict__ out, size_t n) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n) {
    float r = rho[i];
    out[i] = p[i] / (r * r);
  }
}

void *Model::pack_buffer(Group *g, std::string const &kind, size_t item_bytes, std::vector<uint64_t> const &key,
                         bool &stale, cudaStream_t s) {
  PackEntry &e = packs_[{g, kind}];
  size_t n = std::max<size_t>(g->count, 1);
  if (e.cap < n || e.item_bytes != item_bytes) {
    if (e.d) PG_CUDA(cudaFreeAsync(e.d, s));
    PG_CUDA(cudaMallocAsync(&e.d, n * item_bytes, s));
    e.cap = n;
    e.item_bytes = item_bytes;
    e.key.clear();
  }
  stale = e.key != key;
  return e.d;
}

void Model::pack_commit(Group *g, std::string const &kind, std::vector<uint64_t> const &key) {
  packs_[{g, kind}].key = key;
}

static std::vector<uint64_t> vkey(std::initializer_list<VaryingField const *> fs, size_t n) {
  std::vector<uint64_t> k{uint64_t(n)};
  for (auto *f : fs) {
    k.push_back(reinterpret_cast<uint64_t>(f->d));
    k.push_back(f->version);
  }
  return k;
}

float4 const *Model::packed_xs(Group *g, VaryingField *x, VaryingField *sc, char const *kind, cudaStream_t s) {
  auto key = vkey({x, sc}, g->count);
  bool stale = false;
  auto *out = static_cast<float4 *>(pack_buffer(g, kind, 16, key, stale, s));
  if (stale && g->count) {
    k_pack_xs<<<div_up(g->count, 256), 256, 0, s>>>(static_cast<float4 const *>(x->d), static_cast<float const *>(sc->d),
                                                    out, g->count); count_launch();
    PG_LAUNCH_CHECK();
  }
  pack_commit(g, kind, key);
  return out;
}

float4 const *Model::packed_xmr(Group *g, VaryingField *x, VaryingField *m, VaryingField *rho, cudaStream_t s) {
  auto key = vkey({x, m, rho}, g->count);
  bool stale = false;
  auto *out = static_cast<float4 *>(pack_buffer(g, "xmr", 16, key, stale, s));
  if (stale && g->count) {
    k_pack_xmr<<<div_up(g->count, 256), 256, 0, s>>>(static_cast<float4 const *>(x->d), static_cast<float const *>(m->d),
                                                     static_cast<float const *>(rho->d), out, g->count); count_launch();
    PG_LAUNCH_CHECK();
  }
  pack_commit(g, "xmr", key);
  return out;
}

size_t Model::device_bytes() const {
  size_t b = arena_cap_;
  for (auto const &kv : groups_)
    for (auto const &f : kv.second->varying)
      b += f.second.cap * (f.second.type.is_vec3() ? 16 : f.second.type.host_item_bytes());
  for (auto const &kv : packs_) b += kv.second.cap * kv.second.item_bytes;
  return b;
}

float *Model::pr_buffer(Group *g, cudaStream_t s) {
  bool stale = false;
  return static_cast<float *>(pack_buffer(g, "pr", 4, {}, stale, s));
}

float const *Model::packed_pr(Group *g, VaryingField *p, VaryingField *rho, cudaStream_t s) {
  auto key = vkey({p, rho}, g->count);
  bool stale = false;
  auto *out = static_cast<float *>(pack_buffer(g, "pr", 4, key, stale, s));
  if (stale && g->count) {
    k_pack_pr<<<div_up(g->count, 256), 256, 0, s>>>(static_cast<float const *>(p->d), static_cast<float const *>(rho->d),
                                                    out, g->count); count_launch();
    PG_LAUNCH_CHECK();
  }
  pack_commit(g, "pr", key);
  return out;
}

// ---------------------------------------------------------------------------
// Model
// ---------------------------------------------------------------------------

Model::Model() {
  PG_CUDA(cudaStreamCreateWithFlags(&stream_, cudaStreamNonBlocking));
  arena_cap_ = 64 * 1024;
  PG_CUDA(cudaMalloc(&arena_d_, arena_cap_));
  PG_CUDA(cudaMemset(arena_d_, 0, arena_cap_));
  PG_CUDA(cudaMalloc(&red_d, 3 * 4096 * sizeof(double)));
  PG_CUDA(cudaMalloc(&red_count_d, 64 * sizeof(unsigned)));
  PG_CUDA(cudaMemset(red_count_d, 0, 64 * sizeof(unsigned)));
  PG_CUDA(cudaMalloc(&scalars_d, 64 * sizeof(double)));
  PG_CUDA(cudaMemset(scalars_d, 0, 64 * sizeof(double)));
  PG_CUDA(cudaMalloc(&status_d, 16 * sizeof(int)));
  PG_CUDA(cudaMemset(status_d, 0, 16 * sizeof(int)));
  PG_CUDA(cudaMalloc(&stats_d, 16 * sizeof(double)));
  stats_reset(stream_);
  PG_CUDA(cudaStreamSynchronize(stream_));
}

Model::~Model() {
  cudaStreamSynchronize(stream_);
  for (auto &kv : packs_)
    if (kv.second.d) cudaFree(kv.second.d);
  for (auto &g : groups_)
    for (auto &kv : g.second->varying)
      if (kv.second.d) cudaFree(kv.second.d);
  cudaFree(arena_d_);
  cudaFree(red_d);
  cudaFree(red_count_d);
  cudaFree(scalars_d);
  cudaFree(status_d);
  cudaFree(stats_d);
  cudaStreamDestroy(stream_);
}

void Model::reindex() {
  int i = 0;
  for (auto &kv : groups_) kv.second->index = i++;
}

Group &Model::add_group(std::string const &name, std::string const &type) {
  if (name.empty()) throw Error("invalid group name");
  auto it = groups_.find(name);
  if (it != groups_.end()) {
    if (it->second->type != type) throw Error("group of different type already exists: " + name);
    return *it->second;
  }
  if (groups_.size() >= size_t(kMaxGroups)) throw Error("too many groups (at most 16)");
  auto &g = groups_[name];
  g.reset(new Group(this, name, type));
  reindex();
  layout_version++;
  return *g;
}

Group *Model::find_group(std::string const &name) {
  auto it = groups_.find(name);
  return it == groups_.end() ? nullptr : it->second.get();
}

Group &Model::group(std::string const &name) {
  auto *g = find_group(name);
  if (!g) throw Error("group does not exist: " + name);
  return *g;
}

std::vector<Group *> Model::groups_by_index() {
  std::vector<Group *> r;
  for (auto &kv : groups_) r.push_back(kv.second.get());
  return r;
}

SmallField &Model::alloc_small(SmallField &f, FieldType const &t) {
  size_t bytes = (t.host_item_bytes() + 15) / 16 * 16;
  if (arena_used_ + bytes > arena_cap_) throw Error("uniform/global field arena exhausted");
  f.type = t;
  f.offset = arena_used_;
  arena_used_ += bytes;
  return f;
}

SmallField &Model::add_global(std::string const &name, FieldType const &t) {
  auto it = global_.find(name);
  if (it != global_.end()) {
    if (it->second.type != t) throw Error("global field of different type already exists: " + name);
    return it->second;
  }
  SmallField &f = global_[name];
  return alloc_small(f, t);
}

SmallField *Model::find_global(std::string const &name) {
  auto it = global_.find(name);
  return it == global_.end() ? nullptr : &it->second;
}

void Model::small_set(SmallField const &f, void const *host, cudaStream_t s) {
  PG_CUDA(cudaMemcpyAsync(small_ptr(f), host, f.type.host_item_bytes(), cudaMemcpyHostToDevice, s));
  PG_CUDA(cudaStreamSynchronize(s));
}

struct Words16 {
  uint32_t w[16];
};
__global__ void k_set_words(uint32_t *dst, Words16 v, int n) {
  int i = threadIdx.x;
  if (i < n) dst[i] = v.w[i];
}

void Model::small_set_async(SmallField const &f, void const *host, cudaStream_t s) {
  size_t bytes = f.type.host_item_bytes();
  if (bytes > sizeof(Words16)) {
    small_set(f, host, s);
    return;
  }
  Words16 v{};
  std::memcpy(v.w, host, bytes);
  k_set_words<<<1, 32, 0, s>>>(static_cast<uint32_t *>(small_ptr(f)), v, int(bytes / 4)); count_launch();
  PG_LAUNCH_CHECK();
}

__global__ void k_stats_reset(double *st) {
  int i = threadIdx.x;
  if (i < 16) st[i] = (i == 3) ? -INFINITY : 0.0;
}
void Model::stats_reset(cudaStream_t s) {
  k_stats_reset<<<1, 32, 0, s>>>(stats_d); count_launch();
  PG_LAUNCH_CHECK();
}

void Model::small_get(SmallField const &f, void *host, cudaStream_t s) {
  PG_CUDA(cudaMemcpyAsync(host, small_ptr(f), f.type.host_item_bytes(), cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
}

} // namespace prtcl_gpu
