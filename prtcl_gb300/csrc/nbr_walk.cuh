// Device-side walk over the neighbour lists of one item (the lists of
// nhood.hpp), shared by the hand-written schemes and by schemes generated
// from the scheme language.
#pragma once

#include "nhood.hpp"

namespace prtcl_gpu {

// neighbour entries a sweep thread holds at a time (16 or 8; measured per
// sweep on the 1M dam break)
constexpr uint32_t kNbrBatchDefault = 16;

struct NbrList {
  unsigned char const *chunks; // 96-byte chunks (16 offsets + 16 factors), chunk c of item i at (c * n + i)
  uint32_t const *idx32;       // [i * cap + k]: j (read for wide items only)
  uint2 const *cb;             // per item: (count | kWide, base)
  uint32_t cap;                // row length in entries, a multiple of 16
  uint32_t n;                  // rows
};

// Calls f(j, factor) for the neighbours of item i, in list order.  A chunk
// of 16 entries is fetched with six 16-byte streaming loads (evict-first:
// the lists are read once per sweep, the gathered particle records should
// stay in L2), so that its 16 gathers can be in flight together.
// (keep_l2: plain L2-cached loads instead, for a row that is walked again
// right after)
template <uint32_t kNbrBatch = kNbrBatchDefault, class F>
__device__ __forceinline__ void for_each_nbr(NbrList const &L, uint32_t i, bool with_gf, F &&f, bool keep_l2 = false) {
  uint2 cb = __ldg(L.cb + i);
  uint32_t c = min(cb.x & ~kWide, L.cap);
  bool wide = (cb.x & kWide) != 0;
  unsigned char const *row = L.chunks + size_t(i) * kChunkBytes;
  // entries are taken kNbrBatch at a time (16: a whole chunk; 8: half a
  // chunk, fewer registers held per thread).  Measured per sweep on the 1M
  // dam break: 8 is faster for the pressure acceleration, the WKBB18
  // diagonal and system product; 16 for the density and pressure sweeps.
  for (uint32_t kb = 0; kb < c; kb += kNbrBatch) {
    uint32_t h = (kb % kChunk) / kNbrBatch; // batch within the chunk
    uint4 const *ch = reinterpret_cast<uint4 const *>(row + size_t(kb / kChunk) * L.n * kChunkBytes);
    uint32_t j[kNbrBatch];
    if (wide) {
      uint4 const *w32 = reinterpret_cast<uint4 const *>(L.idx32 + size_t(i) * L.cap + kb);
#pragma unroll
      for (int v = 0; v < int(kNbrBatch / 4); ++v) {
        uint4 a = __ldcs(w32 + v);
        j[4 * v] = a.x;
        j[4 * v + 1] = a.y;
        j[4 * v + 2] = a.z;
        j[4 * v + 3] = a.w;
      }
    } else {
#pragma unroll
      for (int v = 0; v < int(kNbrBatch / 8); ++v) {
        uint4 a = keep_l2 ? __ldcg(ch + h * (kNbrBatch / 8) + v) : __ldcs(ch + h * (kNbrBatch / 8) + v);
        uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
        for (int t = 0; t < 4; ++t) {
          // signed 16-bit offsets from the row's base
          j[8 * v + 2 * t] = cb.y + uint32_t(int32_t(int16_t(w[t] & 0xFFFFu)));
          j[8 * v + 2 * t + 1] = cb.y + uint32_t(int32_t(w[t]) >> 16);
        }
      }
    }
    float g[kNbrBatch];
    if (with_gf) {
#pragma unroll
      for (int v = 0; v < int(kNbrBatch / 4); ++v) {
        uint4 const *gp = ch + 2 + h * (kNbrBatch / 4) + v;
        uint4 a = keep_l2 ? __ldcg(gp) : __ldcs(gp);
        g[4 * v] = __uint_as_float(a.x);
        g[4 * v + 1] = __uint_as_float(a.y);
        g[4 * v + 2] = __uint_as_float(a.z);
        g[4 * v + 3] = __uint_as_float(a.w);
      }
    } else {
#pragma unroll
      for (int t = 0; t < int(kNbrBatch); ++t) g[t] = 0.0f;
    }
#pragma unroll
    for (int t = 0; t < int(kNbrBatch); ++t)
      if (kb + t < c) f(j[t], g[t]);
  }
}

// Calls f(slot, factor) for the neighbours of item i, in list order, from
// staged lists (nhood.hpp): slot is the neighbour's place among the staged
// items of the item's tile, which the caller has copied to shared memory.
// The slots of chunk c of item i are the 16 halves at (c * n + i) * 16 of
// `slots`; the factors are those of the chunks.
template <uint32_t kNbrBatch = kNbrBatchDefault, class F>
__device__ __forceinline__ void for_each_staged(NbrList const &L, uint16_t const *slots, uint32_t i, F &&f) {
  uint2 cb = __ldg(L.cb + i);
  uint32_t c = min(cb.x & ~kWide, L.cap);
  for (uint32_t kb = 0; kb < c; kb += kNbrBatch) {
    uint32_t h = (kb % kChunk) / kNbrBatch;
    size_t ci = size_t(kb / kChunk) * L.n + i;
    uint4 const *ch = reinterpret_cast<uint4 const *>(L.chunks + ci * kChunkBytes);
    uint4 const *sp = reinterpret_cast<uint4 const *>(slots + ci * kChunk);
    uint32_t sl[kNbrBatch];
#pragma unroll
    for (int v = 0; v < int(kNbrBatch / 8); ++v) {
      uint4 a = __ldcs(sp + h * (kNbrBatch / 8) + v);
      uint32_t w[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
      for (int t = 0; t < 4; ++t) {
        sl[8 * v + 2 * t] = w[t] & 0xFFFFu;
        sl[8 * v + 2 * t + 1] = w[t] >> 16;
      }
    }
    float g[kNbrBatch];
#pragma unroll
    for (int v = 0; v < int(kNbrBatch / 4); ++v) {
      uint4 a = __ldcs(ch + 2 + h * (kNbrBatch / 4) + v);
      g[4 * v] = __uint_as_float(a.x);
      g[4 * v + 1] = __uint_as_float(a.y);
      g[4 * v + 2] = __uint_as_float(a.z);
      g[4 * v + 3] = __uint_as_float(a.w);
    }
#pragma unroll
    for (int t = 0; t < int(kNbrBatch); ++t)
      if (kb + t < c) f(sl[t], g[t]);
  }
}

} // namespace prtcl_gpu
