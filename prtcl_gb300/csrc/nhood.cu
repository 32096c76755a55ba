// Device uniform-grid neighbourhood (see nhood.hpp for the algorithm).
#include "nhood.hpp"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cooperative_groups.h>
#include <cstring>
#include <limits>

namespace prtcl_gpu {

namespace {

constexpr uint32_t kFull = 0xffffffffu;

// the 13 half-stencil offsets (util/grouped_uniform_grid.hpp:52-68)
__constant__ int c_offsets[13][3] = {{1, 0, 0},  {0, 1, 0},   {0, 0, 1},  {1, 1, 0},  {1, 0, 1},
                                     {0, 1, 1},  {1, 1, 1},   {0, -1, 1}, {1, 0, -1}, {1, 1, -1},
                                     {1, -1, -1}, {1, -1, 0}, {1, -1, 1}};

// ---------------------------------------------------------------------------
// key helpers
// ---------------------------------------------------------------------------

__host__ __device__ __forceinline__ uint32_t unsign(int32_t i) { return uint32_t(i) + 0x7FFFFFFFu; }

// gather the bits of u selected by mask into the low bits (software PEXT)
__host__ __device__ __forceinline__ uint32_t pext32(uint32_t u, uint32_t mask) {
  uint32_t r = 0;
  int k = 0;
  while (mask) {
    uint32_t low = mask & (~mask + 1u);
    if (u & low) r |= (1u << k);
    ++k;
    mask &= mask - 1u;
  }
  return r;
}

// spread the low 21 bits of x to every third bit of a 64-bit word
__host__ __device__ __forceinline__ uint64_t spread3(uint32_t x) {
  uint64_t v = x & 0x1fffffu;
  v = (v | v << 32) & 0x1f00000000ffffULL;
  v = (v | v << 16) & 0x1f0000ff0000ffULL;
  v = (v | v << 8) & 0x100f00f00f00f00fULL;
  v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
  v = (v | v << 2) & 0x1249249249249249ULL;
  return v;
}

// pext32(u, k.keep) from the runs of `keep` (the same bits; a run's bits
// keep their order and the runs are packed from bit 0 up)
__device__ __forceinline__ uint32_t key_pext(uint32_t u, KeyInfo const &k) {
  if (k.nruns == 0) return pext32(u, k.keep);
  uint32_t r = 0;
#pragma unroll
  for (int t = 0; t < kKeyRuns; ++t)
    if (t < k.nruns) r |= (u & k.run_mask[t]) >> k.run_shift[t];
  return r;
}

__device__ __forceinline__ uint64_t make_key(uint32_t u0, uint32_t u1, uint32_t u2, KeyInfo const &k) {
  return (spread3(key_pext(u0, k)) << 2) | (spread3(key_pext(u1, k)) << 1) | spread3(key_pext(u2, k));
}

// is u consistent with the deleted bit positions (could a cell have it?)
__host__ __device__ __forceinline__ bool key_valid(uint32_t u, KeyInfo const &k) {
  uint32_t b = u >> 31;
  uint32_t t = u ^ (b ? 0xFFFFFFFFu : 0u);
  if (t & k.rel_eq) return false;
  if (~t & k.rel_ne) return false;
  if (!(k.keep & 0x80000000u) && ((u & 0x80000000u) != k.b31_const)) return false;
  return true;
}

// (int32) floor((double) x / radius) (util/grouped_uniform_grid.hpp:621-632).
// FP32 fast path: t = x * (1/radius) is within 2^-22.4 |t| of x / radius, so
// floor(t) is exact unless t lies within that distance of an integer; then
// (near cell faces) the FP64 division decides.  GB300's FP64 rate is a small
// fraction of its FP32 rate.
__device__ __forceinline__ int32_t axis_gi(float x, float rinv, double radius) {
  float t = x * rinv;
  float f = floorf(t);
  float d = t - f;
  float near = fminf(d, 1.0f - d);
  if (near > fabsf(t) * 4.76837158203125e-07f + 1e-30f) return int32_t(f);
  return int32_t(floor(double(x) / radius));
}
__device__ __forceinline__ int3 x_to_gi(float4 x, GridView const &gv) {
  return make_int3(axis_gi(x.x, gv.rinv, gv.radius), axis_gi(x.y, gv.rinv, gv.radius),
                   axis_gi(x.z, gv.rinv, gv.radius));
}

__device__ __forceinline__ uint64_t seg_key(GridView const &gv, uint32_t seg) {
  return gv.seg_shift < 64 ? (uint64_t(seg) << gv.seg_shift) : 0ull;
}
__device__ __forceinline__ uint32_t item_seg(GridView const &gv, int g, uint32_t i) {
  return gv.seg[g] ? uint32_t(gv.seg[g][i]) : 0u;
}

__device__ __forceinline__ int find_cell(GridView const &gv, int3 gi, uint32_t seg) {
  uint32_t u0 = unsign(gi.x), u1 = unsign(gi.y), u2 = unsign(gi.z);
  if (!key_valid(u0, gv.key) || !key_valid(u1, gv.key) || !key_valid(u2, gv.key)) return -1;
  uint64_t key = make_key(u0, u1, u2, gv.key) | seg_key(gv, seg);
  int lo = 0, hi = *gv.ncells;
  while (lo < hi) {
    int mid = (lo + hi) >> 1;
    if (gv.cell_key[mid] < key) lo = mid + 1;
    else hi = mid;
  }
  return (lo < *gv.ncells && gv.cell_key[lo] == key) ? lo : -1;
}

// ---------------------------------------------------------------------------
// scans
// ---------------------------------------------------------------------------

template <int NT>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t *sh, uint32_t &total) {
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(kFull, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) sh[w] = x;
  __syncthreads();
  if (w == 0) {
    uint32_t z = lane < NT / 32 ? sh[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, z, o);
      if (lane >= o) z += y;
    }
    if (lane < NT / 32) sh[lane] = z;
  }
  __syncthreads();
  uint32_t pre = (w ? sh[w - 1] : 0u) + x - v;
  total = sh[NT / 32 - 1];
  __syncthreads();
  return pre;
}

// in-place exclusive scan of a short array by one block of 1024 threads
__global__ void k_scan_single(uint32_t *data, size_t len) {
  __shared__ uint32_t sh[32];
  size_t chunk = (len + 1023) / 1024;
  size_t b = threadIdx.x * chunk, e = min(b + chunk, len);
  uint32_t s = 0;
  for (size_t i = b; i < e; ++i) s += data[i];
  uint32_t total;
  uint32_t pre = block_excl_scan<1024>(s, sh, total);
  for (size_t i = b; i < e; ++i) {
    uint32_t v = data[i];
    data[i] = pre;
    pre += v;
  }
}

constexpr int kScanNT = 1024, kScanIPT = 4, kScanTile = kScanNT * kScanIPT;

__global__ void k_scan_reduce(uint32_t const *in, size_t n, uint32_t *sums) {
  __shared__ uint32_t sh[32];
  size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanIPT;
  uint32_t s = 0;
#pragma unroll
  for (int k = 0; k < kScanIPT; ++k)
    if (base + k < n) s += in[base + k];
  uint32_t total;
  block_excl_scan<kScanNT>(s, sh, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

__global__ void k_scan_apply(uint32_t const *in, size_t n, uint32_t const *sums, uint32_t *out) {
  __shared__ uint32_t sh[32];
  size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanIPT;
  uint32_t v[kScanIPT], s = 0;
#pragma unroll
  for (int k = 0; k < kScanIPT; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0u;
    s += v[k];
  }
  uint32_t total;
  uint32_t pre = block_excl_scan<kScanNT>(s, sh, total) + sums[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanIPT; ++k) {
    if (base + k < n) out[base + k] = pre;
    pre += v[k];
  }
}

// ---------------------------------------------------------------------------
// stable LSD radix sort of (uint64 key, uint32 value), 8-bit digits
// ---------------------------------------------------------------------------

constexpr int kRsNT = 256, kRsWarps = kRsNT / 32, kRsWarpItems = 256, kRsTile = kRsWarps * kRsWarpItems;

// One pass over the digit of B bits at `shift`: per tile of kRsTile keys a
// histogram (bucket-major, hist[d * tiles + tile]), then after its exclusive
// scan a stable scatter that ranks equal digits within each warp by lane.
template <int B>
__global__ void k_rs_hist(uint64_t const *__restrict__ keys, size_t n, int shift, uint32_t *hist, uint32_t tiles) {
  constexpr uint32_t NB = 1u << B;
  __shared__ uint32_t h[NB];
  for (uint32_t d = threadIdx.x; d < NB; d += kRsNT) h[d] = 0;
  __syncthreads();
  size_t base = size_t(blockIdx.x) * kRsTile;
  for (int k = 0; k < kRsTile / kRsNT; ++k) {
    size_t i = base + size_t(k) * kRsNT + threadIdx.x;
    if (i < n) atomicAdd(&h[(keys[i] >> shift) & (NB - 1u)], 1u);
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < NB; d += kRsNT) hist[size_t(d) * tiles + blockIdx.x] = h[d];
}

template <int B>
__global__ void k_rs_scatter(uint64_t const *__restrict__ kin, uint32_t const *__restrict__ vin,
                             uint64_t *__restrict__ kout, uint32_t *__restrict__ vout, size_t n, int shift,
                             uint32_t const *__restrict__ offs, uint32_t tiles) {
  constexpr uint32_t NB = 1u << B;
  __shared__ uint32_t cnt[kRsWarps][NB];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (uint32_t d = threadIdx.x; d < kRsWarps * NB; d += kRsNT) cnt[d / NB][d % NB] = 0;
  __syncthreads();
  size_t base = size_t(blockIdx.x) * kRsTile + size_t(w) * kRsWarpItems;
  for (int step = 0; step < kRsWarpItems / 32; ++step) {
    size_t i = base + size_t(step) * 32 + lane;
    uint32_t d = i < n ? uint32_t((kin[i] >> shift) & (NB - 1u)) : NB;
    uint32_t peers = __match_any_sync(kFull, d);
    if (d != NB && lane == __ffs(peers) - 1) cnt[w][d] += __popc(peers);
    __syncwarp();
  }
  __syncthreads();
  for (uint32_t d = threadIdx.x; d < NB; d += kRsNT) {
    uint32_t run = offs[size_t(d) * tiles + blockIdx.x];
    for (int ww = 0; ww < kRsWarps; ++ww) {
      uint32_t c = cnt[ww][d];
      cnt[ww][d] = run;
      run += c;
    }
  }
  __syncthreads();
  uint32_t lt = (1u << lane) - 1u;
  for (int step = 0; step < kRsWarpItems / 32; ++step) {
    size_t i = base + size_t(step) * 32 + lane;
    uint64_t key = 0;
    uint32_t val = 0, d = NB;
    if (i < n) {
      key = kin[i];
      val = vin[i];
      d = uint32_t((key >> shift) & (NB - 1u));
    }
    uint32_t peers = __match_any_sync(kFull, d);
    uint32_t pos = (d != NB) ? cnt[w][d] : 0u;
    __syncwarp();
    if (d != NB) {
      uint32_t dst = pos + __popc(peers & lt);
      kout[dst] = key;
      vout[dst] = val;
      if (lane == __ffs(peers) - 1) cnt[w][d] = pos + __popc(peers);
    }
    __syncwarp();
  }
}

// The same stable LSD sort for small grids in one launch of a thread-block
// cluster, over 8-bit digits: CTA r of the cluster holds sorted positions
// [r M, (r + 1) M) in shared memory (keys and values, two buffers).  Per
// pass every CTA ranks its items by digit as k_rs_scatter does (per-warp
// counts, ranks within a warp by lane), publishes its digit totals, and
// after a cluster barrier each item's new position is the cluster-wide
// start of its digit, plus the totals of that digit in the CTAs before, plus
// its rank in the CTA; it is stored straight into the owning CTA's shared
// memory.  A second barrier ends the pass.  The order is the tiled sort's:
// by digit, then by position before the pass.
constexpr int kRcNT = 1024, kRcWarps = kRcNT / 32;
constexpr uint32_t kRcMaxPerCta = 8000; // 24 bytes per item + 32 KB of counters fit 227 KB
__global__ void __launch_bounds__(kRcNT, 1) k_rs_cluster(uint64_t const *__restrict__ kin,
                                                         uint32_t const *__restrict__ vin, uint64_t *kout,
                                                         uint32_t *vout, uint32_t N, uint32_t M, int total_bits) {
  namespace cg = cooperative_groups;
  cg::cluster_group cl = cg::this_cluster();
  uint32_t r = cl.block_rank(), C = cl.num_blocks();
  extern __shared__ __align__(16) unsigned char rc_smem[];
  uint64_t *ka = reinterpret_cast<uint64_t *>(rc_smem), *kb = ka + M;
  uint32_t *va = reinterpret_cast<uint32_t *>(kb + M), *vb = va + M;
  uint32_t(*cnt)[256] = reinterpret_cast<uint32_t(*)[256]>(vb + M); // [kRcWarps][256]
  __shared__ uint32_t tot[256], base[256], wsum[8];
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t lo = r * M, nl = lo < N ? min(M, N - lo) : 0u;
  for (uint32_t i = threadIdx.x; i < nl; i += kRcNT) {
    ka[i] = kin[lo + i];
    va[i] = vin[lo + i];
  }
  // warp w ranks the local items [w * wi, (w + 1) * wi)
  uint32_t wi = (M + kRcWarps - 1) / kRcWarps;
  wi = (wi + 31u) & ~31u;
  uint32_t w0 = min(nl, uint32_t(w) * wi), w1 = min(nl, w0 + wi);
  uint32_t lt = (1u << lane) - 1u;
  for (int shift = 0; shift < total_bits; shift += 8) {
    for (uint32_t d = threadIdx.x; d < kRcWarps * 256u; d += kRcNT) cnt[d / 256][d % 256] = 0u;
    __syncthreads();
    for (uint32_t b = w0; b < w1; b += 32) {
      uint32_t i = b + lane;
      uint32_t d = i < w1 ? uint32_t((ka[i] >> shift) & 0xFFu) : 256u;
      uint32_t peers = __match_any_sync(kFull, d);
      if (d != 256u && lane == __ffs(peers) - 1) cnt[w][d] += __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    // per digit: exclusive offsets over the warps, the CTA's total
    if (threadIdx.x < 256) {
      uint32_t d = threadIdx.x, run = 0;
      for (int ww = 0; ww < kRcWarps; ++ww) {
        uint32_t c = cnt[ww][d];
        cnt[ww][d] = run;
        run += c;
      }
      tot[d] = run;
    }
    cl.sync(); // every CTA's totals are complete
    // cluster-wide totals per digit, their exclusive scan over the digits,
    // and the totals of this digit in the CTAs before this one
    uint32_t T = 0, before = 0;
    if (threadIdx.x < 256) {
      for (uint32_t q = 0; q < C; ++q) {
        uint32_t t = *cl.map_shared_rank(&tot[threadIdx.x], q);
        T += t;
        if (q < r) before += t;
      }
      uint32_t x = T;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
      }
      if (lane == 31) wsum[w] = x;
      base[threadIdx.x] = x - T + before; // exclusive within the warp's 32 digits
    }
    __syncthreads();
    if (threadIdx.x < 256) {
      uint32_t add = 0;
      for (int ww = 0; ww < w; ++ww) add += wsum[ww];
      base[threadIdx.x] += add;
    }
    __syncthreads();
    for (uint32_t b = w0; b < w1; b += 32) {
      uint32_t i = b + lane;
      uint64_t key = 0;
      uint32_t val = 0, d = 256u;
      if (i < w1) {
        key = ka[i];
        val = va[i];
        d = uint32_t((key >> shift) & 0xFFu);
      }
      uint32_t peers = __match_any_sync(kFull, d);
      uint32_t pos = d != 256u ? base[d] + cnt[w][d] : 0u;
      __syncwarp();
      if (d != 256u) {
        uint32_t dst = pos + __popc(peers & lt);
        uint32_t q = dst / M, li = dst - q * M;
        *cl.map_shared_rank(kb + li, q) = key;
        *cl.map_shared_rank(vb + li, q) = val;
        if (lane == __ffs(peers) - 1) cnt[w][d] += __popc(peers);
      }
      __syncwarp();
    }
    cl.sync(); // every item has landed; the totals may be reused
    uint64_t *tk = ka;
    ka = kb;
    kb = tk;
    uint32_t *tv = va;
    va = vb;
    vb = tv;
  }
  for (uint32_t i = threadIdx.x; i < nl; i += kRcNT) {
    kout[lo + i] = ka[i];
    vout[lo + i] = va[i];
  }
}

// ---------------------------------------------------------------------------
// grid build kernels
// ---------------------------------------------------------------------------

struct PosTable {
  float4 const *pos[kMaxGroups];
};

__device__ __forceinline__ int group_of(uint32_t const *goff, int G, uint32_t n) {
  int g = 0;
  while (g + 1 < G && n >= goff[g + 1]) ++g;
  return g;
}

// pass 1: per item in group-major order, the biased grid indices and the
// handle; OR-reductions of the bit statistics that select the key bits
// (grid-stride; the OR of the block is committed with one atomic per word,
// so that the atomics on the four shared words do not serialise the pass).
// KEY: the key layout of the previous update is taken (it is confirmed
// against these statistics before the grid is read), so the pass writes the
// Z-order keys themselves (the work of k_cells_key) instead of the indices.
constexpr int kCellsUNT = 256;
template <bool KEY>
__global__ void __launch_bounds__(kCellsUNT) k_cells_u(const __grid_constant__ PosTable pt, GridView gv, int G, size_t N, uint32_t *ukeys,
                                                       uint64_t *keys, uint32_t *vals, uint32_t *stats) {
  __shared__ uint32_t sh[4][kCellsUNT / 32];
  uint32_t ne = 0, eq = 0, a1 = 0, a0 = 0;
  for (size_t n = blockIdx.x * size_t(blockDim.x) + threadIdx.x; n < N; n += size_t(gridDim.x) * blockDim.x) {
    int g = group_of(gv.goff, G, uint32_t(n));
    uint32_t i = uint32_t(n) - gv.goff[g];
    int3 gi = x_to_gi(pt.pos[g][i], gv);
    uint32_t u[3] = {unsign(gi.x), unsign(gi.y), unsign(gi.z)};
    for (int a = 0; a < 3; ++a) {
      uint32_t t = u[a] ^ ((u[a] >> 31) ? 0xFFFFFFFFu : 0u);
      ne |= t;
      eq |= ~t;
      a1 |= u[a] & 0x80000000u;
      a0 |= ~u[a] & 0x80000000u;
    }
    if constexpr (KEY)
      keys[n] = make_key(u[0], u[1], u[2], gv.key) | seg_key(gv, item_seg(gv, g, i));
    else
      reinterpret_cast<uint4 *>(ukeys)[n] = make_uint4(u[0], u[1], u[2], 0u);
    vals[n] = (uint32_t(g) << 28) | i;
  }
  ne = __reduce_or_sync(kFull, ne);
  eq = __reduce_or_sync(kFull, eq);
  a1 = __reduce_or_sync(kFull, a1);
  a0 = __reduce_or_sync(kFull, a0);
  int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[0][w] = ne;
    sh[1][w] = eq;
    sh[2][w] = a1;
    sh[3][w] = a0;
  }
  __syncthreads();
  if (threadIdx.x < 4) {
    uint32_t v = 0;
    for (int k = 0; k < kCellsUNT / 32; ++k) v |= sh[threadIdx.x][k];
    if (v) atomicOr(&stats[threadIdx.x], v);
  }
}

__global__ void k_cells_key(uint32_t const *ukeys, uint32_t const *vals, size_t N, GridView gv, uint64_t *keys) {
  size_t n = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (n < N) {
    uint4 u = reinterpret_cast<uint4 const *>(ukeys)[n];
    uint32_t h = vals[n];
    keys[n] = make_key(u.x, u.y, u.z, gv.key) | seg_key(gv, item_seg(gv, int(h >> 28), h & 0x0FFFFFFFu));
  }
}

// The cells from the sorted keys in three launches: per tile of kScanTile
// sorted items the number of cell starts (k_cf_count, an item starts a cell
// where its key differs from its predecessor's), their exclusive scan over
// the tiles (k_scan_single), then every item's cell and the cell tables
// (k_cf_fill).  A thread holds kScanIPT consecutive items.
__global__ void __launch_bounds__(kScanNT) k_cf_count(uint64_t const *__restrict__ keys, size_t N, uint32_t *sums) {
  __shared__ uint32_t sh[32];
  size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanIPT;
  uint32_t f = 0;
  if (base < N) {
    uint64_t prev = base > 0 ? keys[base - 1] : 0ull;
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k)
      if (base + k < N) {
        uint64_t key = keys[base + k];
        f += (base + k == 0 || key != prev) ? 1u : 0u;
        prev = key;
      }
  }
  uint32_t total;
  block_excl_scan<kScanNT>(f, sh, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// excl_tiles: the exclusive scan of k_cf_count's sums; cell(s) is the
// number of cell starts at or before s, minus one
__global__ void __launch_bounds__(kScanNT) k_cf_fill(const __grid_constant__ PosTable pt, GridView gv, uint64_t const *__restrict__ keys,
                                                     uint32_t const *__restrict__ vals, uint32_t const *excl_tiles,
                                                     size_t N, int32_t *s2c, int32_t *r2s, int32_t *cell_start,
                                                     uint64_t *cell_key, int4 *cell_gi, int *ncells,
                                                     int32_t *cell_adj) {
  __shared__ uint32_t sh[32];
  size_t base = size_t(blockIdx.x) * kScanTile + size_t(threadIdx.x) * kScanIPT;
  uint64_t key[kScanIPT];
  uint32_t fl[kScanIPT], f = 0;
  if (base < N) {
    uint64_t prev = base > 0 ? keys[base - 1] : 0ull;
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
      key[k] = base + k < N ? keys[base + k] : 0ull;
      fl[k] = base + k < N && (base + k == 0 || key[k] != prev) ? 1u : 0u;
      prev = key[k];
      f += fl[k];
    }
  } else {
#pragma unroll
    for (int k = 0; k < kScanIPT; ++k) {
      key[k] = 0ull;
      fl[k] = 0u;
    }
  }
  uint32_t total;
  uint32_t run = block_excl_scan<kScanNT>(f, sh, total) + excl_tiles[blockIdx.x];
#pragma unroll
  for (int k = 0; k < kScanIPT; ++k) {
    size_t si = base + k;
    if (si >= N) break;
    run += fl[k];
    int32_t c = int32_t(run) - 1;
    s2c[si] = c;
    uint32_t h = vals[si];
    uint32_t g = h >> 28, i = h & 0x0FFFFFFFu;
    r2s[gv.goff[g] + i] = int32_t(si);
    if (fl[k]) {
      cell_start[c] = int32_t(si);
      cell_key[c] = key[k];
      int3 gi = x_to_gi(pt.pos[g][i], gv);
      cell_gi[c] = make_int4(gi.x, gi.y, gi.z, 0);
      // no neighbour yet (the adjacency kernel fills the slots it finds)
      // (a cell's 26 slots start at a multiple of 104 bytes: 8-byte stores)
      int2 *a = reinterpret_cast<int2 *>(cell_adj + size_t(c) * 26);
      for (int q = 0; q < 13; ++q) a[q] = make_int2(-1, -1);
    }
    if (si == N - 1) {
      cell_start[c + 1] = int32_t(N);
      *ncells = c + 1;
    }
  }
}

// The cell with key kt, searched from cell c (key kc != kt) outwards: a
// galloping search towards kt, then a binary search in the bracket found.
// Adjacent cells are mostly near in Z-order, so the probes stay close to c.
__device__ __forceinline__ int find_from(uint64_t const *__restrict__ keys, int C, int c, uint64_t kc, uint64_t kt) {
  int lo, hi;
  if (kt > kc) {
    lo = c + 1;
    int step = 1, probe = c + 1;
    while (probe < C && keys[probe] < kt) {
      lo = probe + 1;
      step <<= 1;
      probe = c + step;
    }
    hi = min(probe, C);
  } else {
    hi = c;
    int step = 1, probe = c - 1;
    while (probe >= 0 && keys[probe] > kt) {
      hi = probe;
      step <<= 1;
      probe = c - step;
    }
    lo = max(probe, 0);
  }
  while (lo < hi) { // first index in [lo, hi) with key >= kt
    int mid = (lo + hi) >> 1;
    if (keys[mid] < kt) lo = mid + 1;
    else hi = mid;
  }
  return (lo < C && keys[lo] == kt) ? lo : -1;
}

// 26-cell adjacency (util/grouped_uniform_grid.hpp:312-337): cell c searches
// the cells at +offset[k] only and writes both mirror slots, adj[c][k] = d
// and adj[d][25 - k] = c, so every slot is written by exactly one thread
// (adj starts at -1)
// Hash table of the cell keys (open addressing, linear probing) for the
// adjacency lookups: a power-of-two table larger than the item count, so it
// always has an empty slot (every probe loop ends); the slot of a key does
// not depend on the order of insertion, so the lookups are exact.
// kEmptyKey marks an empty slot; no cell key equals it while the keys use
// fewer than 64 bits (the host falls back to the searches otherwise).
constexpr uint64_t kEmptyKey = ~0ull;
__device__ __forceinline__ uint32_t key_hash(uint64_t k, uint32_t mask) {
  return uint32_t((k * 0x9E3779B97F4A7C15ull) >> 32) & mask;
}
__global__ void k_hash_insert(GridView gv, size_t N, uint64_t *hk, int32_t *hv, uint32_t mask) {
  size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  int C = *gv.ncells;
  if (c >= N || int(c) >= C) return;
  uint64_t key = gv.cell_key[c];
  uint32_t h = key_hash(key, mask);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    unsigned long long prev = atomicCAS(reinterpret_cast<unsigned long long *>(hk + h), kEmptyKey, key);
    if (prev == kEmptyKey) {
      hv[h] = int32_t(c);
      return;
    }
    h = (h + 1) & mask;
  }
}
__device__ __forceinline__ int hash_find(uint64_t const *__restrict__ hk, int32_t const *__restrict__ hv, uint32_t mask,
                                         uint64_t key) {
  uint32_t h = key_hash(key, mask);
  for (uint32_t probe = 0; probe <= mask; ++probe) {
    uint64_t k = hk[h];
    if (k == key) return hv[h];
    if (k == kEmptyKey) return -1;
    h = (h + 1) & mask;
  }
  return -1;
}

// (hk == nullptr: galloping searches over the sorted cell keys instead)
__global__ void k_cells_adj(GridView gv, int4 const *cell_gi, size_t N, int32_t *adj, uint64_t const *hk,
                            int32_t const *hv, uint32_t mask) {
  size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  int C = *gv.ncells;
  if (c >= N || int(c) >= C) return;
  int4 g = cell_gi[c];
  uint64_t kc = gv.cell_key[c];
  uint64_t sk = seg_key(gv, gv.seg_shift < 64 ? uint32_t(kc >> gv.seg_shift) : 0u);
  for (int k = 0; k < 13; ++k) {
    int3 p = make_int3(g.x + c_offsets[k][0], g.y + c_offsets[k][1], g.z + c_offsets[k][2]);
    uint32_t u0 = unsign(p.x), u1 = unsign(p.y), u2 = unsign(p.z);
    if (!key_valid(u0, gv.key) || !key_valid(u1, gv.key) || !key_valid(u2, gv.key)) continue;
    uint64_t kt = make_key(u0, u1, u2, gv.key) | sk;
    int d = hk ? hash_find(hk, hv, mask, kt) : find_from(gv.cell_key, C, int(c), kc, kt);
    if (d >= 0) {
      adj[c * 26 + k] = d;
      adj[size_t(d) * 26 + 25 - k] = int32_t(c);
    }
  }
}

// The same adjacency through the hash table, with the 13 lookups of a cell
// in flight together: every home slot is read first, then the values of the
// slots that hold their key; a lookup whose home slot holds another key
// continues with the probe loop of hash_find.  The slots found are those of
// hash_find, so the adjacency is the same.
__global__ void __launch_bounds__(128) k_cells_adj_hash(GridView gv, int4 const *cell_gi, size_t N, int32_t *adj,
                                                        uint64_t const *__restrict__ hk,
                                                        int32_t const *__restrict__ hv, uint32_t mask) {
  size_t c = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  int C = *gv.ncells;
  if (c >= N || int(c) >= C) return;
  int4 g = cell_gi[c];
  uint64_t kc = gv.cell_key[c];
  uint64_t sk = seg_key(gv, gv.seg_shift < 64 ? uint32_t(kc >> gv.seg_shift) : 0u);
  uint64_t kt[13], got[13];
  uint32_t slot[13], valid = 0;
#pragma unroll
  for (int k = 0; k < 13; ++k) {
    int3 p = make_int3(g.x + c_offsets[k][0], g.y + c_offsets[k][1], g.z + c_offsets[k][2]);
    uint32_t u0 = unsign(p.x), u1 = unsign(p.y), u2 = unsign(p.z);
    bool ok = key_valid(u0, gv.key) && key_valid(u1, gv.key) && key_valid(u2, gv.key);
    kt[k] = ok ? (make_key(u0, u1, u2, gv.key) | sk) : kEmptyKey;
    slot[k] = key_hash(kt[k], mask);
    valid |= ok ? (1u << k) : 0u;
  }
#pragma unroll
  for (int k = 0; k < 13; ++k) got[k] = (valid >> k) & 1u ? hk[slot[k]] : kEmptyKey;
  int d[13];
#pragma unroll
  for (int k = 0; k < 13; ++k) d[k] = ((valid >> k) & 1u) && got[k] == kt[k] ? hv[slot[k]] : -1;
#pragma unroll
  for (int k = 0; k < 13; ++k) {
    if (!((valid >> k) & 1u)) continue;
    if (got[k] != kt[k] && got[k] != kEmptyKey) d[k] = hash_find(hk, hv, mask, kt[k]);
    if (d[k] >= 0) {
      adj[c * 26 + k] = d[k];
      adj[size_t(d[k]) * 26 + 25 - k] = int32_t(c);
    }
  }
}

__global__ void k_xsorted(const __grid_constant__ PosTable pt, uint32_t const *vals, size_t N, float4 *xs) {
  size_t s = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (s < N) {
    uint32_t h = vals[s];
    float4 x = pt.pos[h >> 28][h & 0x0FFFFFFFu];
    x.w = __uint_as_float(h);
    xs[s] = x;
  }
}

constexpr int kBuildNT = 128; // query items (threads) per list-build block
#ifndef PRTCL_PAIRED_APPEND
#define PRTCL_PAIRED_APPEND 1
#endif

struct ListOut {
  unsigned char *chunks[kMaxListGroups];
  uint16_t *slots[kMaxListGroups]; // staged lists: each entry's staged slot
  uint2 *tile_info, *tile_cells;   // staged lists: per tile (see nhood.hpp)
  uint32_t *idx32[kMaxListGroups];
  uint32_t cap[kMaxListGroups];
  uint2 *cb;        // [G][n]
  uint32_t *maxcnt; // [kMaxListGroups]: the longest row of each group
  uint32_t n;
  int G;
  int with_gf; // factors are written (lists built without them never read them)
};

// State of one item's list towards one neighbour group.  The current chunk
// is buffered in shared memory (24 words per thread and group: 8 words of
// packed 16-bit deltas, 16 factor words; word w of thread t at
// buf[(g * 24 + w) * NT + t]) and written as six 16-byte stores when full.
// Deltas are signed, relative to the row's first neighbour j0 (the row's
// base); a row whose neighbours do not all fit becomes "wide": its indices
// then go to idx32 (the entries already written are converted on the spot).
// A wide row's offset words are never read, so the 8 words hold its 32-bit
// indices instead, one half-chunk at a time, written to idx32 as two 16-byte
// stores when the half is full: one whole sector per 8 entries rather than a
// sector per entry (neighbours of an unpermuted group make nearly every row
// wide).
struct RowState {
  uint32_t c, j0;
  bool wide;
};

// BW: buffered words per thread and group: 24 (8 of packed offsets, 16 of
// factors), or 32 for staged lists (8 more of packed slots)
template <int BW> __device__ __forceinline__ uint32_t &bufw(uint32_t *buf, int g, int w) {
  return buf[(size_t(g) * BW + w) * kBuildNT + threadIdx.x];
}

template <int BW>
__device__ __forceinline__ void flush_chunk(ListOut const &lo, int g, uint32_t i, uint32_t chunk, bool wide,
                                            uint32_t *buf) {
  size_t ci = size_t(chunk) * lo.n + i;
  uint4 *dst = reinterpret_cast<uint4 *>(lo.chunks[g] + ci * kChunkBytes);
  // offsets (2 vectors, not for a wide row), then the factors (4 vectors)
  // when the lists carry them: sweeps read factors only from lists built
  // with a smoothing scale
  int v0 = wide ? 2 : 0, nv = lo.with_gf ? 6 : 2;
  for (int v = v0; v < nv; ++v)
    dst[v] = make_uint4(bufw<BW>(buf, g, 4 * v), bufw<BW>(buf, g, 4 * v + 1), bufw<BW>(buf, g, 4 * v + 2),
                        bufw<BW>(buf, g, 4 * v + 3));
  if (BW == 32) {
    uint4 *sd = reinterpret_cast<uint4 *>(lo.slots[g] + ci * kChunk);
    for (int v = 0; v < 2; ++v)
      sd[v] = make_uint4(bufw<BW>(buf, g, 24 + 4 * v), bufw<BW>(buf, g, 25 + 4 * v), bufw<BW>(buf, g, 26 + 4 * v),
                         bufw<BW>(buf, g, 27 + 4 * v));
  }
}

// the 8 buffered indices of a wide row's entries e0..e0+7 (e0 % 8 == 0) to
// idx32: 32 aligned bytes (cap is a multiple of 16)
template <int BW>
__device__ __forceinline__ void flush_wide_half(ListOut const &lo, int g, uint32_t i, uint32_t e0, uint32_t *buf) {
  uint4 *dst = reinterpret_cast<uint4 *>(lo.idx32[g] + size_t(i) * lo.cap[g] + e0);
  dst[0] = make_uint4(bufw<BW>(buf, g, 0), bufw<BW>(buf, g, 1), bufw<BW>(buf, g, 2), bufw<BW>(buf, g, 3));
  dst[1] = make_uint4(bufw<BW>(buf, g, 4), bufw<BW>(buf, g, 5), bufw<BW>(buf, g, 6), bufw<BW>(buf, g, 7));
}

template <int BW>
__device__ __forceinline__ void row_add(ListOut const &lo, int g, uint32_t i, RowState &R, uint32_t j, float f,
                                        uint32_t slot16, uint32_t *buf) {
  uint32_t k = R.c++;
  if (k >= lo.cap[g]) return; // overflow: the host grows the lists and builds again
  if (k == 0) R.j0 = j;
  int32_t d = int32_t(j - R.j0);
  uint32_t slot = k % kChunk;
  if (!R.wide && (d < -32768 || d > 32767)) {
    // becomes wide: entries 0..k-1 to idx32 (full chunks from global memory,
    // the current one from the buffer)
    R.wide = true;
    for (uint32_t e = 0; e < k; ++e) {
      uint32_t w;
      if (e / kChunk == k / kChunk) w = bufw<BW>(buf, g, int((e % kChunk) / 2));
      else w = reinterpret_cast<uint32_t const *>(lo.chunks[g] + (size_t(e / kChunk) * lo.n + i) * kChunkBytes)[(e % kChunk) / 2];
      int32_t de = int32_t(int16_t((e & 1) ? (w >> 16) : (w & 0xFFFFu)));
      lo.idx32[g][size_t(i) * lo.cap[g] + e] = R.j0 + uint32_t(de);
    }
    // the current half-chunk's entries back into the buffer as indices (the
    // packed words they came from are no longer needed)
    for (uint32_t e = k - slot % 8; e < k; ++e) bufw<BW>(buf, g, int(e % 8)) = lo.idx32[g][size_t(i) * lo.cap[g] + e];
  }
  if (R.wide) {
    bufw<BW>(buf, g, int(slot % 8)) = j;
  } else {
    // the slot's half-word (little-endian: even slots low); a stale upper
    // half past the row's end is cleared when the last chunk is written
    reinterpret_cast<uint16_t *>(&bufw<BW>(buf, g, int(slot / 2)))[slot & 1] = uint16_t(uint32_t(d) & 0xFFFFu);
  }
  if (lo.with_gf) bufw<BW>(buf, g, 8 + int(slot)) = __float_as_uint(f);
  if (BW == 32) reinterpret_cast<uint16_t *>(&bufw<BW>(buf, g, 24 + int(slot / 2)))[slot & 1] = uint16_t(slot16);
  if (R.wide && slot % 8 == 7) flush_wide_half<BW>(lo, g, i, k - 7, buf);
  if (slot == kChunk - 1) flush_chunk<BW>(lo, g, i, k / kChunk, R.wide, buf);
}

// cbase (staged lists, BW == 32): the cell's first slot among the tile's
// staged items, so that the hit at sorted index s has slot cbase + (s - s0)
template <int NG, int BW>
__device__ __forceinline__ void visit_cell(GridView const &gv, float4 const *__restrict__ xs, int cell, f3 xi,
                                           uint32_t i, ListOut const &lo, RowState *R, KernelParams const &K,
                                           bool with_gf, uint32_t *buf, uint32_t cbase = 0u) {
  if (cell < 0) return;
  int s0 = gv.cell_start[cell], s1 = gv.cell_start[cell + 1];
  // the distance tests of up to 32 candidates into a mask, then the
  // accepted ones appended in candidate order: the append code runs once
  // per hit of the lane with the most hits in the cell, not once per
  // candidate on which any lane of the warp hits
  for (int base = s0; base < s1; base += 32) {
    int e = min(s1 - base, 32);
    uint32_t mask = 0;
    if constexpr (NG == 1) {
      // one neighbour group (the search): four tests in flight (measured
      // faster there; slower with two groups and factors)
#pragma unroll 4
      for (int t = 0; t < e; ++t) {
        float d2 = nsq3(sub3(xi, mk3(xs[base + t])));
        if (d2 < gv.r2lt) mask |= 1u << t; // == (double) d2 < r^2
      }
    } else {
      for (int t = 0; t < e; ++t) {
        float d2 = nsq3(sub3(xi, mk3(xs[base + t])));
        if (d2 < gv.r2lt) mask |= 1u << t;
      }
    }
    while (mask) {
      int t = __ffs(int(mask)) - 1;
      mask &= mask - 1u;
      float4 xj = xs[base + t];
      uint32_t h = __float_as_uint(xj.w);
      uint32_t g = h >> 28, j = h & 0x0FFFFFFFu;
      float f = with_gf ? kgrad_factor(K, nsq3(sub3(xi, mk3(xj)))) : 0.0f;
      uint32_t slot16 = BW == 32 ? cbase + uint32_t(base + t - s0) : 0u;
#pragma unroll
      for (int q = 0; q < NG; ++q)
        if (q == int(g)) row_add<BW>(lo, q, i, R[q], j, f, slot16, buf);
    }
  }
}

// The test half of visit_cell for a cell of at most 32 items: the hits as a
// mask over the cell's items from s0 (0 for no cell)
__device__ __forceinline__ uint32_t cell_mask(GridView const &gv, float4 const *__restrict__ xs, int cell, f3 xi,
                                              int &s0, int &e) {
  uint32_t mask = 0;
  s0 = 0;
  e = 0;
  if (cell < 0) return 0u;
  s0 = gv.cell_start[cell];
  e = gv.cell_start[cell + 1] - s0;
  if (e > 32) return 0u;
  for (int t = 0; t < e; ++t) {
    float d2 = nsq3(sub3(xi, mk3(xs[s0 + t])));
    if (d2 < gv.r2lt) mask |= 1u << t;
  }
  return mask;
}
// the append half of visit_cell for the hit at sorted index s
template <int NG, int BW>
__device__ __forceinline__ void append_hit(float4 const *__restrict__ xs, int s, f3 xi, uint32_t i, ListOut const &lo,
                                           RowState *R, KernelParams const &K, bool with_gf, uint32_t *buf) {
  float4 xj = xs[s];
  uint32_t h = __float_as_uint(xj.w);
  uint32_t g = h >> 28, j = h & 0x0FFFFFFFu;
  float f = with_gf ? kgrad_factor(K, nsq3(sub3(xi, mk3(xj)))) : 0.0f;
#pragma unroll
  for (int q = 0; q < NG; ++q)
    if (q == int(g)) row_add<BW>(lo, q, i, R[q], j, f, 0u, buf);
}

// Lower bounds, in units of the cell edge (= the radius), of the distance
// from a point to the faces of its own cell: lo to the lower face (the cells
// at offset -1 along the axis), hi to the upper face (offset +1).  t = x / r
// in FP32 is within |t| 2^-22.4 of the exact quotient; where that error could
// put the point on the other side of a face, both bounds are 0.
// Returns false (bounds 0) unless the point lies, beyond that error, inside
// the cell of index `gi` along the axis (the cell the grid assigned to it).
__device__ __forceinline__ bool face_bounds(float x, float rinv, int gi, float &lo, float &hi) {
  float t = x * rinv;
  float f = floorf(t);
  float d = t - f;
  float err = fabsf(t) * 4.8e-7f + 1e-6f;
  lo = 0.0f;
  hi = 0.0f;
  if (!(fminf(d, 1.0f - d) > 2.0f * err) || !(fabsf(f) < 2.0e9f) || int(f) != gi) return false;
  lo = fmaxf(d - err, 0.0f);
  hi = fmaxf((1.0f - d) - err, 0.0f);
  return true;
}

// neighbour lists of one query group (grid query of util/grouped_uniform_grid.hpp:407-531)
// `order` (optional): thread t builds the row of item order[t] (the group's
// items in grid order), so that the threads of a warp walk nearby cells.
// Adjacent cells whose box is farther than the radius from the query (with a
// margin of 1e-4 of the radius, far above the rounding of the exact test)
// cannot hold a neighbour and are not scanned; the lists are unchanged.
// With one or two neighbour groups (24.6 KB of row buffers per block at
// most) nine blocks fit an SM's shared memory; holding the registers to
// that (56) took the 1M dam break's list build from 604 to 585 µs.
// Staged lists: the tile's staged cells (the cells adjacent to its items'
// cells, own cell included) in an open-addressing table of kStageHash
// slots, their first staged slots, and the tile's table in global memory
// (nhood.hpp).  All threads of the block take part; returns whether the
// tile's staged items fit (kStageCap items, kStageCells cells).
__device__ __forceinline__ uint32_t stage_hash(int c) { return (uint32_t(c) * 2654435761u) >> 23; } // 9 bits
static_assert(kStageHash == 512, "stage_hash yields 9 bits");

__device__ __forceinline__ int stage_find(int const *hkey, int c) {
  uint32_t h = stage_hash(c);
  for (uint32_t probe = 0; probe < kStageHash; ++probe) {
    uint32_t sl = (h + probe) & (kStageHash - 1);
    if (hkey[sl] == c) return int(sl);
  }
  return -1;
}

__device__ bool stage_tile(GridView const &gv, int home, bool has, uint32_t tile, ListOut const &lo, int *hkey,
                           uint32_t *hbase) {
  __shared__ int homes[kBuildNT];
  __shared__ uint32_t wsum[kBuildNT / 32], wocc[kBuildNT / 32];
  __shared__ int over;
  for (uint32_t sl = threadIdx.x; sl < kStageHash; sl += kBuildNT) hkey[sl] = -1;
  if (threadIdx.x == 0) over = 0;
  homes[threadIdx.x] = home;
  __syncthreads();
  // the first item of each run of equal home cells enters the run's 27 cells
  if (has && (threadIdx.x == 0 || homes[threadIdx.x - 1] != home)) {
    for (int k = -1; k < 26; ++k) {
      int c = k < 0 ? home : gv.cell_adj[size_t(home) * 26 + k];
      if (c < 0) continue;
      uint32_t h = stage_hash(c);
      bool placed = false;
      for (uint32_t probe = 0; probe < kStageHash && !placed; ++probe) {
        int old = atomicCAS(&hkey[(h + probe) & (kStageHash - 1)], -1, c);
        placed = old == -1 || old == c;
      }
      if (!placed) over = 1;
    }
  }
  __syncthreads();
  // the staged items of each table slot; slots in (thread, m) order
  constexpr int M = kStageHash / kBuildNT;
  uint32_t cnt[M], mine = 0, occ = 0;
#pragma unroll
  for (int m = 0; m < M; ++m) {
    int c = hkey[threadIdx.x + m * kBuildNT];
    cnt[m] = c >= 0 ? uint32_t(gv.cell_start[c + 1] - gv.cell_start[c]) : 0u;
    mine += cnt[m];
    occ += c >= 0 ? 1u : 0u;
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  uint32_t incl = mine, oincl = occ;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t v = __shfl_up_sync(0xffffffffu, incl, o), vo = __shfl_up_sync(0xffffffffu, oincl, o);
    if (lane >= o) {
      incl += v;
      oincl += vo;
    }
  }
  if (lane == 31) {
    wsum[w] = incl;
    wocc[w] = oincl;
  }
  __syncthreads();
  uint32_t off = incl - mine, u = oincl - occ, total = 0, ncells = 0;
  for (int k = 0; k < int(kBuildNT / 32); ++k) {
    if (k < w) {
      off += wsum[k];
      u += wocc[k];
    }
    total += wsum[k];
    ncells += wocc[k];
  }
  if (total > kStageCap || ncells > kStageCells) over = 1;
  __syncthreads();
  bool fit = over == 0;
  if (fit) {
#pragma unroll
    for (int m = 0; m < M; ++m) {
      uint32_t sl = threadIdx.x + m * kBuildNT;
      int c = hkey[sl];
      if (c >= 0) {
        hbase[sl] = off;
        lo.tile_cells[size_t(tile) * kStageCells + u] = make_uint2(uint32_t(gv.cell_start[c]), off);
        off += cnt[m];
        ++u;
      }
    }
  }
  if (threadIdx.x == 0) lo.tile_info[tile] = make_uint2(ncells, fit ? total : kNoStage);
  __syncthreads();
  return fit;
}

// neighbour lists of one query group (grid query of util/grouped_uniform_grid.hpp:407-531)
// `order` (optional): thread t builds the row of item order[t] (the group's
// items in grid order), so that the threads of a warp walk nearby cells.
// Adjacent cells whose box is farther than the radius from the query (with a
// margin of 1e-4 of the radius, far above the rounding of the exact test)
// cannot hold a neighbour and are not scanned; the lists are unchanged.
// With one or two neighbour groups (24.6 KB of row buffers per block at
// most) nine blocks fit an SM's shared memory; holding the registers to
// that (56) took the 1M dam break's list build from 604 to 585 µs.
// STAGE: staged lists (a group in cell order, no `order`): the block is the
// tile of items it builds, and every entry also gets its staged slot.
template <int NG, bool STAGE>
__global__ void __launch_bounds__(kBuildNT, STAGE ? 5 : (NG <= 2 ? 9 : 1))
    k_build_lists(GridView gv, float4 const *__restrict__ xs, float4 const *__restrict__ qpos, int q, ListOut lo,
                  float const *hp, float *hcache, uint32_t const *__restrict__ order) {
  constexpr int BW = STAGE ? 32 : 24;
  extern __shared__ uint32_t buf[];
  __shared__ int s_hkey[STAGE ? kStageHash : 1];
  __shared__ uint32_t s_hbase[STAGE ? kStageHash : 1];
  uint32_t t = blockIdx.x * kBuildNT + threadIdx.x;
  bool with_gf = hp != nullptr;
  KernelParams K = kparams(with_gf ? *hp : 1.0f);
  if (t == 0) *hcache = with_gf ? K.h : __int_as_float(0x7fc00000);
  bool staged = false;
  if constexpr (STAGE) {
    bool has = t < lo.n;
    int home = has ? gv.s2c[gv.r2s[gv.goff[q] + t]] : -1;
    staged = stage_tile(gv, home, has, blockIdx.x, lo, s_hkey, s_hbase);
  }
  if (t >= lo.n) return;
  uint32_t i = order ? order[t] : t;
  RowState R[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) R[g] = RowState{0u, 0u, false};
  float4 x4 = qpos[i];
  f3 xi = mk3(x4);
  int cell = -1;
  bool fallback = false;
  int3 gi;
  if (gv.in_grid[q]) {
    cell = gv.s2c[gv.r2s[gv.goff[q] + i]];
  } else {
    gi = x_to_gi(x4, gv);
    cell = find_cell(gv, gi, item_seg(gv, q, i));
    fallback = cell < 0;
  }
  // the staged base of a visited cell (0 where the tile is not staged: the
  // slots are then never read)
  auto cbase = [&](int c) -> uint32_t {
    if (!STAGE || !staged || c < 0) return 0u;
    int sl = stage_find(s_hkey, c);
    return sl >= 0 ? s_hbase[sl] : 0u;
  };
  if (!fallback) {
    float lo3[3], hi3[3];
    int4 cg = gv.cell_gi[cell];
    bool inside = face_bounds(x4.x, gv.rinv, cg.x, lo3[0], hi3[0]);
    inside = face_bounds(x4.y, gv.rinv, cg.y, lo3[1], hi3[1]) && inside;
    inside = face_bounds(x4.z, gv.rinv, cg.z, lo3[2], hi3[2]) && inside;
    if (!inside)
      for (int a = 0; a < 3; ++a) lo3[a] = hi3[a] = 0.0f;
#if PRTCL_PAIRED_APPEND
    if constexpr (!STAGE && NG == 2) {
      // the visit sequence (own cell, slots 0..25) two cells at a time: both
      // cells tested, then the hits of both appended in one loop, so that
      // the loop runs as often as the lane with the most hits in the pair
      // (not in each cell); a cell of more than 32 items is visited whole.
      // With two groups and gradient factors the append is most of the
      // work: 1M dam break 590 -> 571 us, 256 scenes 9.05 -> 8.73 ms per
      // step.  The one-group search keeps the cell-by-cell walk, whose
      // test loop keeps four candidates in flight (clustered points, with
      // many cells of more than 32 items, lost 7 % paired).
      auto slot_cell = [&](int v) -> int {
        if (v == 0) return cell;
        int k = v - 1;
        // slot k < 13: +offset[k]; slot 25 - k: -offset[k]
        int kk = k < 13 ? k : 25 - k;
        int sg = k < 13 ? 1 : -1;
        float lb = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          int o = sg * c_offsets[kk][a];
          float b = o > 0 ? hi3[a] : (o < 0 ? lo3[a] : 0.0f);
          lb += b * b;
        }
        return lb > 1.0001f ? -1 : gv.cell_adj[size_t(cell) * 26 + k];
      };
      for (int v = 0; v < 27; v += 2) {
        int ca = slot_cell(v), cb = v + 1 < 27 ? slot_cell(v + 1) : -1;
        int sa, ea, sb, eb;
        uint32_t ma = cell_mask(gv, xs, ca, xi, sa, ea), mb = cell_mask(gv, xs, cb, xi, sb, eb);
        if (ea > 32) {
          visit_cell<NG, BW>(gv, xs, ca, xi, i, lo, R, K, with_gf, buf);
          ma = 0u;
        }
        if (eb > 32) {
          // A's hits first, then B whole
          while (ma) {
            int t = __ffs(int(ma)) - 1;
            ma &= ma - 1u;
            append_hit<NG, BW>(xs, sa + t, xi, i, lo, R, K, with_gf, buf);
          }
          visit_cell<NG, BW>(gv, xs, cb, xi, i, lo, R, K, with_gf, buf);
          mb = 0u;
        }
        while (ma | mb) {
          int s;
          if (ma) {
            int t = __ffs(int(ma)) - 1;
            ma &= ma - 1u;
            s = sa + t;
          } else {
            int t = __ffs(int(mb)) - 1;
            mb &= mb - 1u;
            s = sb + t;
          }
          append_hit<NG, BW>(xs, s, xi, i, lo, R, K, with_gf, buf);
        }
      }
    } else
#endif
    {
      visit_cell<NG, BW>(gv, xs, cell, xi, i, lo, R, K, with_gf, buf, cbase(cell));
      for (int k = 0; k < 26; ++k) {
        // slot k < 13: +offset[k]; slot 25 - k: -offset[k]
        int kk = k < 13 ? k : 25 - k;
        int sg = k < 13 ? 1 : -1;
        float lb = 0.0f;
#pragma unroll
        for (int a = 0; a < 3; ++a) {
          int o = sg * c_offsets[kk][a];
          float b = o > 0 ? hi3[a] : (o < 0 ? lo3[a] : 0.0f);
          lb += b * b;
        }
        if (lb > 1.0001f) continue;
        int c = gv.cell_adj[size_t(cell) * 26 + k];
        visit_cell<NG, BW>(gv, xs, c, xi, i, lo, R, K, with_gf, buf, cbase(c));
      }
    }
  } else {
    uint32_t sq = item_seg(gv, q, i);
    for (int k = 0; k < 13; ++k) {
      int3 p = make_int3(gi.x + c_offsets[k][0], gi.y + c_offsets[k][1], gi.z + c_offsets[k][2]);
      visit_cell<NG, BW>(gv, xs, find_cell(gv, p, sq), xi, i, lo, R, K, with_gf, buf);
      int3 m = make_int3(gi.x - c_offsets[k][0], gi.y - c_offsets[k][1], gi.z - c_offsets[k][2]);
      visit_cell<NG, BW>(gv, xs, find_cell(gv, m, sq), xi, i, lo, R, K, with_gf, buf);
    }
  }
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    if (g >= lo.G) break;
    uint32_t n = R[g].c;
    lo.cb[size_t(g) * lo.n + i] = make_uint2(n | (R[g].wide ? kWide : 0u), R[g].j0);
    {
      // the longest row, one atomic per warp: the host grows the lists when
      // it exceeds the capacity (the rows past it were cut) and shrinks them
      // when it is far below
      unsigned am = __activemask();
      uint32_t wmax = __reduce_max_sync(am, n);
      if (int(threadIdx.x & 31u) == __ffs(int(am)) - 1) atomicMax(&lo.maxcnt[g], wmax);
    }
    if (n > lo.cap[g]) {
      // overflow: the row is rebuilt after the host grows the lists
    } else if (n % kChunk) {
      // the partial last chunk (and half-chunk of a wide row), zero-filled
      bool wide = R[g].wide;
      if (wide && n % 8) {
        for (uint32_t e = n % 8; e < 8; ++e) bufw<BW>(buf, g, int(e)) = 0u;
        flush_wide_half<BW>(lo, g, i, n - n % 8, buf);
      }
      for (uint32_t slot = n % kChunk; slot < kChunk; ++slot) {
        if (!wide) {
          uint32_t &w = bufw<BW>(buf, g, int(slot / 2));
          w = (slot & 1) ? (w & 0xFFFFu) : 0u;
        }
        bufw<BW>(buf, g, 8 + int(slot)) = 0u;
        if (BW == 32) {
          uint32_t &w = bufw<BW>(buf, g, 24 + int(slot / 2));
          w = (slot & 1) ? (w & 0xFFFFu) : 0u;
        }
      }
      flush_chunk<BW>(lo, g, i, n / kChunk, wide, buf);
    }
  }
}

// Lists of a small query group (the list_split knob): kSplit threads per
// query, each walking a contiguous part of the query's visit sequence (own
// cell, then adjacency slots 0..25: parts of 7, 7, 7 and 6 cells), so that
// a query's dependent chain of cell walks is a quarter as long.  A first
// walk counts each part's neighbours per group (with the first index and
// the index range); the query's threads combine them by shuffles into each
// row's count, base index and wide / narrow form, and a second walk writes
// every entry straight to its place in the chunks (or idx32 for a wide
// row), with its gradient factor.  The visited cells, the distance test and
// the factor arithmetic are those of k_build_lists, so the rows are the
// same entry for entry; the tail of a row's last chunk is zero-filled as
// there.  For a query group of the grid (no fallback search).
constexpr int kSplit = 4, kSplitNT = 128;
constexpr size_t kSplitMaxQueries = 65536;
__device__ __forceinline__ int split_first_visit(int sub) { return sub * 7; } // 0, 7, 14, 21; 27 at the end

template <class F>
__device__ __forceinline__ void split_walk(GridView const &gv, float4 const *__restrict__ xs, int cell,
                                           float const *lo3, float const *hi3, int v0, int v1, f3 xi, F &&f) {
  for (int v = v0; v < v1; ++v) {
    int c = cell;
    if (v > 0) {
      int k = v - 1;
      // slot k < 13: +offset[k]; slot 25 - k: -offset[k]
      int kk = k < 13 ? k : 25 - k;
      int sg = k < 13 ? 1 : -1;
      float lb = 0.0f;
#pragma unroll
      for (int a = 0; a < 3; ++a) {
        int o = sg * c_offsets[kk][a];
        float b = o > 0 ? hi3[a] : (o < 0 ? lo3[a] : 0.0f);
        lb += b * b;
      }
      if (lb > 1.0001f) continue;
      c = gv.cell_adj[size_t(cell) * 26 + k];
    }
    if (c < 0) continue;
    int s0 = gv.cell_start[c], s1 = gv.cell_start[c + 1];
    for (int base = s0; base < s1; base += 32) {
      int e = min(s1 - base, 32);
      uint32_t mask = 0;
      for (int t = 0; t < e; ++t) {
        float d2 = nsq3(sub3(xi, mk3(xs[base + t])));
        if (d2 < gv.r2lt) mask |= 1u << t;
      }
      while (mask) {
        int t = __ffs(int(mask)) - 1;
        mask &= mask - 1u;
        f(base + t);
      }
    }
  }
}

template <int NG>
__global__ void __launch_bounds__(kSplitNT) k_build_lists_split(GridView gv, float4 const *__restrict__ xs,
                                                               float4 const *__restrict__ qpos, int q, ListOut lo,
                                                               float const *hp, float *hcache,
                                                               uint32_t const *__restrict__ order) {
  uint32_t gt = blockIdx.x * kSplitNT + threadIdx.x;
  uint32_t t = gt / kSplit;
  int sub = int(gt % kSplit);
  bool with_gf = hp != nullptr;
  KernelParams K = kparams(with_gf ? *hp : 1.0f);
  if (gt == 0) *hcache = with_gf ? K.h : __int_as_float(0x7fc00000);
  bool active = t < lo.n; // the same for a query's kSplit threads (one warp holds whole queries)
  uint32_t i = active ? (order ? order[t] : t) : 0u;
  f3 xi = {0.0f, 0.0f, 0.0f};
  int cell = -1;
  float lo3[3] = {0.0f, 0.0f, 0.0f}, hi3[3] = {0.0f, 0.0f, 0.0f};
  if (active) {
    float4 x4 = qpos[i];
    xi = mk3(x4);
    cell = gv.s2c[gv.r2s[gv.goff[q] + i]];
    int4 cg = gv.cell_gi[cell];
    bool inside = face_bounds(x4.x, gv.rinv, cg.x, lo3[0], hi3[0]);
    inside = face_bounds(x4.y, gv.rinv, cg.y, lo3[1], hi3[1]) && inside;
    inside = face_bounds(x4.z, gv.rinv, cg.z, lo3[2], hi3[2]) && inside;
    if (!inside)
      for (int a = 0; a < 3; ++a) lo3[a] = hi3[a] = 0.0f;
  }
  int v0 = split_first_visit(sub), v1 = sub + 1 < kSplit ? split_first_visit(sub + 1) : 27;
  // 1. per group: hits, the first hit's index, the index range
  uint32_t cnt[NG], first[NG];
  int32_t mn[NG], mx[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    cnt[g] = 0u;
    first[g] = 0u;
    mn[g] = INT32_MAX;
    mx[g] = INT32_MIN;
  }
  if (active)
    split_walk(gv, xs, cell, lo3, hi3, v0, v1, xi, [&](int s) {
      uint32_t h = __float_as_uint(xs[s].w);
      uint32_t g = h >> 28, j = h & 0x0FFFFFFFu;
#pragma unroll
      for (int qq = 0; qq < NG; ++qq)
        if (qq == int(g)) {
          if (cnt[qq] == 0u) first[qq] = j;
          mn[qq] = min(mn[qq], int32_t(j));
          mx[qq] = max(mx[qq], int32_t(j));
          ++cnt[qq];
        }
    });
  // 2. the query's rows: each part's first entry, the count, base and form
  uint32_t pre[NG], total[NG], j0[NG];
  bool wide[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    uint32_t x = cnt[g];
#pragma unroll
    for (int o = 1; o < kSplit; o <<= 1) {
      uint32_t y = __shfl_up_sync(kFull, x, o, kSplit);
      if (sub >= o) x += y;
    }
    pre[g] = x - cnt[g];
    total[g] = __shfl_sync(kFull, x, kSplit - 1, kSplit);
    int src = cnt[g] ? sub : kSplit;
    int32_t lo_j = mn[g], hi_j = mx[g];
#pragma unroll
    for (int o = 1; o < kSplit; o <<= 1) {
      src = min(src, __shfl_xor_sync(kFull, src, o, kSplit));
      lo_j = min(lo_j, __shfl_xor_sync(kFull, lo_j, o, kSplit));
      hi_j = max(hi_j, __shfl_xor_sync(kFull, hi_j, o, kSplit));
    }
    j0[g] = __shfl_sync(kFull, first[g], src < kSplit ? src : 0, kSplit);
    if (src >= kSplit) j0[g] = 0u;
    wide[g] = total[g] > 0u && (hi_j - int32_t(j0[g]) > 32767 || lo_j - int32_t(j0[g]) < -32768);
  }
  if (!active) return;
  // 3. the entries at their places
  uint32_t run[NG];
#pragma unroll
  for (int g = 0; g < NG; ++g) run[g] = pre[g];
  split_walk(gv, xs, cell, lo3, hi3, v0, v1, xi, [&](int s) {
    float4 xj = xs[s];
    uint32_t h = __float_as_uint(xj.w);
    uint32_t g = h >> 28, j = h & 0x0FFFFFFFu;
    float f = with_gf ? kgrad_factor(K, nsq3(sub3(xi, mk3(xj)))) : 0.0f;
#pragma unroll
    for (int qq = 0; qq < NG; ++qq)
      if (qq == int(g)) {
        uint32_t k = run[qq]++;
        if (k < lo.cap[qq]) {
          unsigned char *ch = lo.chunks[qq] + (size_t(k / kChunk) * lo.n + i) * kChunkBytes;
          if (wide[qq]) lo.idx32[qq][size_t(i) * lo.cap[qq] + k] = j;
          else reinterpret_cast<uint16_t *>(ch)[k % kChunk] = uint16_t(uint32_t(int32_t(j - j0[qq])) & 0xFFFFu);
          if (lo.with_gf) reinterpret_cast<uint32_t *>(ch + 32)[k % kChunk] = __float_as_uint(f);
        }
      }
  });
  if (sub != 0) return;
#pragma unroll
  for (int g = 0; g < NG; ++g) {
    if (g >= lo.G) break;
    uint32_t n = total[g];
    lo.cb[size_t(g) * lo.n + i] = make_uint2(n | (wide[g] ? kWide : 0u), j0[g]);
    atomicMax(&lo.maxcnt[g], n);
    if (n > lo.cap[g] || n % kChunk == 0) continue;
    // the partial last chunk (and half-chunk of a wide row), zero-filled
    unsigned char *ch = lo.chunks[g] + (size_t(n / kChunk) * lo.n + i) * kChunkBytes;
    if (wide[g]) {
      for (uint32_t e = n; e % 8; ++e) lo.idx32[g][size_t(i) * lo.cap[g] + e] = 0u;
    } else {
      for (uint32_t slot = n % kChunk; slot < kChunk; ++slot) reinterpret_cast<uint16_t *>(ch)[slot] = 0u;
    }
    if (lo.with_gf)
      for (uint32_t slot = n % kChunk; slot < kChunk; ++slot) reinterpret_cast<uint32_t *>(ch + 32)[slot] = 0u;
  }
}

template <int NG, bool STAGE>
void launch_build_lists(size_t n, size_t smem, cudaStream_t s, GridView const &gv, float4 const *xs,
                        float4 const *qpos, int q, ListOut const &lo, float const *h, float *hcache,
                        uint32_t const *order) {
  PG_CUDA(cudaFuncSetAttribute(k_build_lists<NG, STAGE>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smem)));
  k_build_lists<NG, STAGE><<<div_up(n, kBuildNT), kBuildNT, smem, s>>>(gv, xs, qpos, q, lo, h, hcache, order);
}

__global__ void k_pair_count(uint2 const *cb, size_t n, unsigned long long *total) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  unsigned long long c = (i < n) ? (cb[i].x & ~kWide) : 0u;
  for (int o = 16; o > 0; o >>= 1) c += __shfl_down_sync(kFull, c, o);
  if ((threadIdx.x & 31) == 0 && c) atomicAdd(total, c);
}

__global__ void k_group_flags(uint32_t const *vals, size_t N, uint32_t g, uint32_t *flags) {
  size_t s = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (s < N) flags[s] = ((vals[s] >> 28) == g) ? 1u : 0u;
}

__global__ void k_group_perm(uint32_t const *vals, uint32_t const *flags, uint32_t const *excl, size_t N, uint32_t *perm) {
  size_t s = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (s < N && flags[s]) perm[excl[s]] = vals[s] & 0x0FFFFFFFu;
}

// items of segments that are not due keep their place
__global__ void k_perm_keep(uint16_t const *seg, uint8_t const *due, size_t n, uint32_t *perm) {
  size_t i = blockIdx.x * size_t(blockDim.x) + threadIdx.x;
  if (i < n && !due[seg[i]]) perm[i] = uint32_t(i);
}

} // namespace

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------

// The cluster sort's launch for a grid of N items: 8 CTAs up to
// 8 * kRcMaxPerCta items, 16 (a non-portable cluster size) up to twice that;
// false where N is larger or the device cannot hold such a cluster (probed
// once per device and size with the largest shared-memory footprint).
static bool cluster_sort_config(size_t N, cudaLaunchConfig_t &cfg, cudaLaunchAttribute &attr, uint32_t &M) {
  if (N == 0 || N > 16 * size_t(kRcMaxPerCta)) return false;
  int C = N <= 8 * size_t(kRcMaxPerCta) ? 8 : 16;
  int dev = 0;
  PG_CUDA(cudaGetDevice(&dev));
  // per device and cluster size: 0 unknown, 1 yes, 2 no (models on several
  // host threads may probe at once; every probe of a device finds the same)
  static std::atomic<int> ok[2][64];
  std::atomic<int> &known = ok[C == 16][dev & 63];
  size_t smax = size_t(kRcMaxPerCta) * 24 + size_t(kRcWarps) * 256 * 4;
  M = uint32_t((N + C - 1) / C);
  cfg = cudaLaunchConfig_t{};
  cfg.gridDim = dim3(unsigned(C));
  cfg.blockDim = dim3(unsigned(kRcNT));
  attr = cudaLaunchAttribute{};
  attr.id = cudaLaunchAttributeClusterDimension;
  attr.val.clusterDim.x = unsigned(C);
  attr.val.clusterDim.y = 1;
  attr.val.clusterDim.z = 1;
  cfg.attrs = &attr;
  cfg.numAttrs = 1;
  if (known == 2) return false;
  // the function's attributes belong to the current device's context: set
  // on every call (host-side and cheap), so a new context gets them too
  PG_CUDA(cudaFuncSetAttribute(k_rs_cluster, cudaFuncAttributeMaxDynamicSharedMemorySize, int(smax)));
  if (C > 8) PG_CUDA(cudaFuncSetAttribute(k_rs_cluster, cudaFuncAttributeNonPortableClusterSizeAllowed, 1));
  if (known == 0) {
    cfg.dynamicSmemBytes = smax;
    int clusters = 0;
    cudaError_t e = cudaOccupancyMaxActiveClusters(&clusters, k_rs_cluster, &cfg);
    if (e != cudaSuccess) (void)cudaGetLastError(); // a size the device does not take: no cluster sort
    known.store((e == cudaSuccess && clusters > 0) ? 1 : 2);
  }
  cfg.dynamicSmemBytes = size_t(M) * 24 + size_t(kRcWarps) * 256 * 4;
  return known == 1;
}

static void ensure_sums(size_t nb, uint32_t *&sums, size_t &sums_cap) {
  if (nb > sums_cap) {
    if (sums) PG_CUDA(cudaFree(sums));
    sums_cap = std::max<size_t>(nb, 1024);
    PG_CUDA(cudaMalloc(&sums, sums_cap * sizeof(uint32_t)));
  }
}

static void exclusive_scan(uint32_t const *in, uint32_t *out, size_t n, uint32_t *&sums, size_t &sums_cap,
                           cudaStream_t s) {
  if (n == 0) return;
  size_t nb = (n + kScanTile - 1) / kScanTile;
  ensure_sums(nb, sums, sums_cap);
  k_scan_reduce<<<unsigned(nb), kScanNT, 0, s>>>(in, n, sums); count_launch();
  k_scan_single<<<1, 1024, 0, s>>>(sums, nb); count_launch();
  k_scan_apply<<<unsigned(nb), kScanNT, 0, s>>>(in, n, sums, out); count_launch();
  PG_LAUNCH_CHECK();
}

Nhood::Nhood() {
  PG_CUDA(cudaMalloc(&stats_d_, 16 * sizeof(uint32_t)));
  PG_CUDA(cudaMalloc(&ncells_d_, sizeof(int)));
  PG_CUDA(cudaMemset(ncells_d_, 0, sizeof(int)));
  PG_CUDA(cudaMallocHost(&stats_h_, 16 * sizeof(uint32_t)));
}

static void free_all(std::initializer_list<void *> ps) {
  for (void *p : ps)
    if (p) cudaFree(p);
}

Nhood::~Nhood() {
  for (auto &kv : lists_) free_lists(kv.second);
  free_all({keys_a_, keys_b_, vals_a_, vals_b_, ukeys_, flags_, scan_, r2s_, s2c_, cell_start_, cell_adj_, cell_key_,
            cell_gi_, xsorted_, hist_, block_sums_, stats_d_, ncells_d_, order_, hkeys_, hvals_});
  cudaFreeHost(stats_h_);
}

void Nhood::free_lists(Lists &L) {
  for (int g = 0; g < kMaxGroups; ++g) {
    if (L.idx32[g]) cudaFree(L.idx32[g]);
    if (L.chunks[g]) cudaFree(L.chunks[g]);
    if (L.slots[g]) cudaFree(L.slots[g]);
    L.idx32[g] = nullptr;
    L.chunks[g] = nullptr;
    L.slots[g] = nullptr;
  }
  if (L.tile_info) cudaFree(L.tile_info);
  if (L.tile_cells) cudaFree(L.tile_cells);
  L.tile_info = nullptr;
  L.tile_cells = nullptr;
  L.tile_cap = 0;
  L.staged = false;
  if (L.cb) cudaFree(L.cb);
  if (L.hcache) cudaFree(L.hcache);
  L.cb = nullptr;
  L.hcache = nullptr;
}

// Neighborhood::Load (util/neighborhood.cpp:67-98): remember each group's
// position field (real[3]) and whether it can be a neighbour
void Nhood::load(Model &m) {
  auto gs = m.groups_by_index();
  std::vector<GG> ng(gs.size(), GG{});
  int three = 3;
  FieldType v3 = parse_field_type("f32", 1, &three);
  for (size_t g = 0; g < gs.size(); ++g) {
    ng[g].g = gs[g];
    VaryingField *p = gs[g]->find_varying("position");
    ng[g].pos = (p && p->type == v3) ? p : nullptr;
    ng[g].can_be_neighbor = !gs[g]->has_tag("cannot_be_neighbor");
  }
  // keep the grid of the last Update when the groups and their bindings are
  // unchanged (re-loading schemes and the neighbourhood is routine in the
  // reference's scripts); otherwise it must be updated before use
  bool same = (&m == model_) && ng.size() == gg_.size();
  for (size_t g = 0; same && g < ng.size(); ++g)
    same = ng[g].g == gg_[g].g && ng[g].pos == gg_[g].pos && ng[g].can_be_neighbor == gg_[g].can_be_neighbor;
  model_ = &m;
  gg_ = ng;
  if (!same) {
    has_grid_ = false;
    for (auto &c : permuted_count_) c = 0;
    for (auto &kv : lists_) free_lists(kv.second);
    lists_.clear();
  }
}

void Nhood::ensure_grid_capacity(size_t n) {
  if (n <= cap_) return;
  size_t c = std::max(n + n / 8, size_t(1024));
  free_all({keys_a_, keys_b_, vals_a_, vals_b_, ukeys_, flags_, scan_, r2s_, s2c_, cell_start_, cell_adj_, cell_key_,
            cell_gi_, xsorted_});
  PG_CUDA(cudaMalloc(&keys_a_, c * 8));
  PG_CUDA(cudaMalloc(&keys_b_, c * 8));
  PG_CUDA(cudaMalloc(&vals_a_, c * 4));
  PG_CUDA(cudaMalloc(&vals_b_, c * 4));
  PG_CUDA(cudaMalloc(&ukeys_, c * 16));
  PG_CUDA(cudaMalloc(&flags_, c * 4));
  PG_CUDA(cudaMalloc(&scan_, c * 4));
  PG_CUDA(cudaMalloc(&r2s_, c * 4));
  PG_CUDA(cudaMalloc(&s2c_, c * 4));
  PG_CUDA(cudaMalloc(&cell_start_, (c + 1) * 4));
  PG_CUDA(cudaMalloc(&cell_adj_, c * 26 * 4));
  PG_CUDA(cudaMalloc(&cell_key_, c * 8));
  PG_CUDA(cudaMalloc(&cell_gi_, c * 16));
  PG_CUDA(cudaMalloc(&xsorted_, c * 16));
  cap_ = c;
}

GridView Nhood::view() const {
  GridView v{};
  v.sorted = sorted_vals_;
  v.r2s = r2s_;
  v.s2c = s2c_;
  v.cell_start = cell_start_;
  v.cell_key = cell_key_;
  v.cell_adj = cell_adj_;
  v.cell_gi = cell_gi_;
  v.ncells = ncells_d_;
  for (int g = 0; g <= kMaxGroups; ++g) v.goff[g] = goff_[g];
  for (int g = 0; g < kMaxGroups; ++g) v.in_grid[g] = in_grid_[g];
  for (int g = 0; g < kMaxGroups; ++g) v.seg[g] = (seg_count_ && g < int(seg_.size())) ? seg_[g] : nullptr;
  v.key = key_;
  v.seg_shift = seg_count_ ? 3 * key_.bits : 64;
  v.radius = radius_;
  v.r2 = radius_ * radius_;
  v.rinv = float(1.0 / radius_);
  // the float threshold T with  d2 < T  <=>  (double) d2 < r2
  float a = float(v.r2);
  if (double(a) > v.r2) a = std::nextafter(a, -std::numeric_limits<float>::infinity());
  v.r2lt = (double(a) == v.r2) ? a : std::nextafter(a, std::numeric_limits<float>::infinity());
  return v;
}

// the cell-key layout of the bit statistics ne, eq, a1, a0 of k_cells_u
static KeyInfo key_from_stats(uint32_t const *st) {
  uint32_t ne = st[0], eq = st[1], a1 = st[2], a0 = st[3];
  KeyInfo k{};
  k.keep = ne & eq & 0x7FFFFFFFu;
  k.rel_eq = eq & ~ne & 0x7FFFFFFFu;
  k.rel_ne = ne & ~eq & 0x7FFFFFFFu;
  if (a1 && a0) k.keep |= 0x80000000u;
  else k.b31_const = a1 ? 0x80000000u : 0u;
  k.bits = __builtin_popcount(k.keep);
  key_runs(k);
  return k;
}
static bool same_key(KeyInfo const &a, KeyInfo const &b) {
  return a.keep == b.keep && a.rel_eq == b.rel_eq && a.rel_ne == b.rel_ne && a.b31_const == b.b31_const;
}

void Nhood::settle(cudaStream_t s) {
  if (!key_check_) return;
  PG_CUDA(cudaMemcpyAsync(stats_h_, stats_d_, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  key_check_ = false;
  if (!same_key(key_from_stats(stats_h_), key_)) {
    key_known_ = false;
    update(s);
  }
}

// grouped_uniform_grid::update (util/grouped_uniform_grid.hpp:126-337)
void Nhood::update(cudaStream_t s) {
  if (!model_) throw Error("Neighborhood::Update before Load");
  int G = int(gg_.size());
  PosTable pt{};
  size_t N = 0;
  for (int g = 0; g < kMaxGroups; ++g) in_grid_[g] = 0;
  for (int g = 0; g < G; ++g) {
    goff_[g] = uint32_t(N);
    bool in = gg_[g].pos && gg_[g].can_be_neighbor;
    in_grid_[g] = in ? 1 : 0;
    if (gg_[g].pos) pt.pos[g] = static_cast<float4 const *>(gg_[g].pos->d);
    if (in) {
      if (gg_[g].g->count >= (size_t(1) << 28)) throw Error("group too large for the grid (>= 2^28 items)");
      N += gg_[g].g->count;
    }
  }
  for (int g = G; g <= kMaxGroups; ++g) goff_[g] = uint32_t(N);
  if (N >= (size_t(1) << 31)) throw Error("too many items for the grid");
  N_ = N;
  ensure_grid_capacity(N);
  epoch_++;
  has_grid_ = true;
  if (N == 0) {
    key_check_ = false; // no statistics to confirm
    PG_CUDA(cudaMemsetAsync(ncells_d_, 0, sizeof(int), s));
    sorted_keys_ = keys_a_;
    sorted_vals_ = vals_a_;
    return;
  }
  GridView gv = view();
  // 1. grid indices, handles, bit statistics
  PG_CUDA(cudaMemsetAsync(stats_d_, 0, 16 * sizeof(uint32_t), s));
  unsigned nb = div_up(N, 256);
  {
    ProfScope ps(model_->prof, "grid_keys", s);
    unsigned ub = std::min<unsigned>(div_up(N, kCellsUNT), 152u * 8u);
    if (key_known_) k_cells_u<true><<<ub, kCellsUNT, 0, s>>>(pt, gv, G, N, nullptr, keys_a_, vals_a_, stats_d_);
    else k_cells_u<false><<<ub, kCellsUNT, 0, s>>>(pt, gv, G, N, ukeys_, nullptr, vals_a_, stats_d_);
    count_launch();
  }
  PG_LAUNCH_CHECK();
  KeyInfo k{};
  bool keyed = key_known_; // the keys are written already
  if (key_known_) {
    // the previous update's layout, confirmed before anything reads the grid
    k = key_;
    key_check_ = true;
  } else {
    PG_CUDA(cudaMemcpyAsync(stats_h_, stats_d_, 4 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    k = key_from_stats(stats_h_);
    key_known_ = true;
    key_check_ = false;
  }
  if (k.bits > 21)
    throw Error("grid spans too many cells: " + std::to_string(k.bits) +
                " informative bits per axis (at most 21 are supported)");
  if (seg_count_ && 3 * k.bits + seg_bits_ > 64)
    throw Error("grid spans too many cells for " + std::to_string(seg_count_) + " segments: " +
                std::to_string(k.bits) + " informative bits per axis");
  key_ = k;
  gv = view();
  // 2. compressed Z-order keys (segment above them)
  model_->prof.begin("grid_sort", s);
  if (!keyed) {
    k_cells_key<<<nb, 256, 0, s>>>(ukeys_, vals_a_, N, gv, keys_a_); count_launch();
    PG_LAUNCH_CHECK();
  }
  // 3. stable LSD radix sort over the informative bits
  int total_bits = 3 * k.bits + (seg_count_ ? seg_bits_ : 0);
  uint64_t *kin = keys_a_, *kout = keys_b_;
  uint32_t *vin = vals_a_, *vout = vals_b_;
  uint32_t tiles = uint32_t((N + kRsTile - 1) / kRsTile);
  // the fewest passes of at most 10-bit digits, the digits as even as possible
  int passes = std::max(1, (total_bits + 9) / 10);
  int dbits = std::max(8, (total_bits + passes - 1) / passes);
  size_t hl = size_t(tiles) << dbits;
  if (hl > hist_cap_) {
    if (hist_) PG_CUDA(cudaFree(hist_));
    hist_cap_ = hl + hl / 4;
    PG_CUDA(cudaMalloc(&hist_, hist_cap_ * 4));
  }
  cudaLaunchConfig_t rc_cfg;
  cudaLaunchAttribute rc_attr;
  uint32_t rc_m = 0;
  bool rc = model_->tune.v[kTuneGridSort] != 0 && cluster_sort_config(N, rc_cfg, rc_attr, rc_m);
  if (rc) {
    rc_cfg.stream = s;
    PG_CUDA(cudaLaunchKernelEx(&rc_cfg, k_rs_cluster, static_cast<uint64_t const *>(kin),
                               static_cast<uint32_t const *>(vin), kout, vout, uint32_t(N), rc_m, total_bits));
    count_launch();
    PG_LAUNCH_CHECK();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  for (int shift = 0; !rc && shift < total_bits; shift += dbits) {
    if (dbits == 8) k_rs_hist<8><<<tiles, kRsNT, 0, s>>>(kin, N, shift, hist_, tiles);
    else if (dbits == 9) k_rs_hist<9><<<tiles, kRsNT, 0, s>>>(kin, N, shift, hist_, tiles);
    else k_rs_hist<10><<<tiles, kRsNT, 0, s>>>(kin, N, shift, hist_, tiles);
    count_launch();
    exclusive_scan(hist_, hist_, hl, block_sums_, block_sums_cap_, s);
    if (dbits == 8) k_rs_scatter<8><<<tiles, kRsNT, 0, s>>>(kin, vin, kout, vout, N, shift, hist_, tiles);
    else if (dbits == 9) k_rs_scatter<9><<<tiles, kRsNT, 0, s>>>(kin, vin, kout, vout, N, shift, hist_, tiles);
    else k_rs_scatter<10><<<tiles, kRsNT, 0, s>>>(kin, vin, kout, vout, N, shift, hist_, tiles);
    count_launch();
    PG_LAUNCH_CHECK();
    std::swap(kin, kout);
    std::swap(vin, vout);
  }
  sorted_keys_ = kin;
  sorted_vals_ = vin;
  gv = view();
  model_->prof.end(s); // grid_sort
  model_->prof.begin("grid_cells", s);
  // 4. cells
  {
    size_t tiles_c = (N + kScanTile - 1) / kScanTile;
    ensure_sums(tiles_c, block_sums_, block_sums_cap_);
    k_cf_count<<<unsigned(tiles_c), kScanNT, 0, s>>>(kin, N, block_sums_); count_launch();
    k_scan_single<<<1, 1024, 0, s>>>(block_sums_, tiles_c); count_launch();
    k_cf_fill<<<unsigned(tiles_c), kScanNT, 0, s>>>(pt, gv, kin, vin, block_sums_, N, s2c_, r2s_, cell_start_,
                                                   cell_key_, cell_gi_, ncells_d_, cell_adj_);
    count_launch();
    PG_LAUNCH_CHECK();
  }
  // 5. adjacency (cells <= N; slots without a neighbour stay -1)
  uint64_t *hk = nullptr;
  int32_t *hv = nullptr;
  uint32_t mask = 0;
  if (total_bits < 64 && N < (size_t(1) << 30)) {
    size_t hs = 1;
    while (hs <= N) hs <<= 1; // > N >= cells: an empty slot always remains
    if (hs > hash_cap_) {
      if (hkeys_) PG_CUDA(cudaFree(hkeys_));
      if (hvals_) PG_CUDA(cudaFree(hvals_));
      PG_CUDA(cudaMalloc(&hkeys_, hs * sizeof(uint64_t)));
      PG_CUDA(cudaMalloc(&hvals_, hs * sizeof(int32_t)));
      hash_cap_ = hs;
    }
    PG_CUDA(cudaMemsetAsync(hkeys_, 0xFF, hs * sizeof(uint64_t), s));
    mask = uint32_t(hs - 1);
    hk = hkeys_;
    hv = hvals_;
    k_hash_insert<<<nb, 256, 0, s>>>(gv, N, hk, hv, mask); count_launch();
  }
  if (hk) k_cells_adj_hash<<<div_up(N, 128), 128, 0, s>>>(gv, cell_gi_, N, cell_adj_, hk, hv, mask);
  else k_cells_adj<<<nb, 256, 0, s>>>(gv, cell_gi_, N, cell_adj_, hk, hv, mask);
  count_launch();
  model_->prof.end(s); // grid_cells
  PG_LAUNCH_CHECK();
}

std::vector<uint64_t> Nhood::pos_versions() const {
  std::vector<uint64_t> v(gg_.size(), 0);
  for (size_t g = 0; g < gg_.size(); ++g)
    v[g] = gg_[g].pos ? (gg_[g].pos->version ^ (uint64_t(gg_[g].g->count) << 40)) : 0;
  return v;
}

bool Nhood::lists_fresh(Lists const &L) const { return L.epoch == epoch_ && L.pos_versions == pos_versions(); }

void Nhood::build_lists(int q, Lists &L, cudaStream_t s, float const *h, bool stage) {
  int G = int(gg_.size());
  if (G > kMaxListGroups) throw Error("neighbour lists support at most 8 groups");
  size_t n = gg_[q].g->count;
  // sorted positions with handles, from the current positions
  PosTable pt{};
  for (int g = 0; g < G; ++g)
    if (gg_[g].pos) pt.pos[g] = static_cast<float4 const *>(gg_[g].pos->d);
  if (N_ > 0) {
    k_xsorted<<<div_up(N_, 256), 256, 0, s>>>(pt, sorted_vals_, N_, xsorted_); count_launch();
    PG_LAUNCH_CHECK();
  }
  // a group that is not in cell order (never permuted, or resized since) is
  // walked in grid order
  uint32_t const *order = nullptr;
  if (in_grid_[q] && n > 0 && permuted_count_[q] != n) {
    if (n > order_cap_) {
      if (order_) PG_CUDA(cudaFree(order_));
      order_cap_ = n + n / 8;
      PG_CUDA(cudaMalloc(&order_, order_cap_ * 4));
    }
    k_group_flags<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, N_, uint32_t(q), flags_); count_launch();
    exclusive_scan(flags_, scan_, N_, block_sums_, block_sums_cap_, s);
    k_group_perm<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, flags_, scan_, N_, order_); count_launch();
    PG_LAUNCH_CHECK();
    order = order_;
  }
  // staged lists: with factors, for a group in cell order, at most two
  // neighbour groups (the staged sweeps' layout)
  bool st = stage && h && in_grid_[q] && !order && G <= 2;
  if (st != L.staged) {
    // a change of form reallocates every list of the group
    for (int g = 0; g < kMaxGroups; ++g) L.cap[g] = 0;
    for (int g = 0; g < kMaxGroups; ++g) {
      if (L.idx32[g]) PG_CUDA(cudaFree(L.idx32[g]));
      if (L.chunks[g]) PG_CUDA(cudaFree(L.chunks[g]));
      if (L.slots[g]) PG_CUDA(cudaFree(L.slots[g]));
      L.idx32[g] = nullptr;
      L.chunks[g] = nullptr;
      L.slots[g] = nullptr;
    }
    L.staged = st;
  }
  // the staged tile tables (after any free_lists() below, which drops them)
  auto ensure_tiles = [&] {
    size_t ntiles = div_up(n, kStageTile);
    if (!st || ntiles <= L.tile_cap) return;
    if (L.tile_info) PG_CUDA(cudaFree(L.tile_info));
    if (L.tile_cells) PG_CUDA(cudaFree(L.tile_cells));
    L.tile_info = nullptr;
    L.tile_cells = nullptr;
    L.tile_cap = 0;
    PG_CUDA(cudaMalloc(&L.tile_info, (ntiles + ntiles / 8 + 1) * sizeof(uint2)));
    PG_CUDA(cudaMalloc(&L.tile_cells, (ntiles + ntiles / 8 + 1) * kStageCells * sizeof(uint2)));
    L.tile_cap = ntiles + ntiles / 8 + 1;
  };
  auto alloc_slots = [&](int g, uint32_t want) {
    if (L.idx32[g]) PG_CUDA(cudaFree(L.idx32[g]));
    if (L.chunks[g]) PG_CUDA(cudaFree(L.chunks[g]));
    if (L.slots[g]) PG_CUDA(cudaFree(L.slots[g]));
    L.idx32[g] = nullptr;
    L.chunks[g] = nullptr;
    L.slots[g] = nullptr;
    if (n > 0) {
      PG_CUDA(cudaMalloc(&L.idx32[g], size_t(want) * n * 4));
      PG_CUDA(cudaMalloc(&L.chunks[g], size_t(want / kChunk) * kChunkBytes * n));
      if (L.staged) PG_CUDA(cudaMalloc(&L.slots[g], size_t(want) * n * sizeof(uint16_t)));
    }
    L.cap[g] = want;
  };
  for (int attempt = 0; attempt < 8; ++attempt) {
    if (L.n != n || !L.cb) {
      free_lists(L);
      for (int g = 0; g < kMaxGroups; ++g) L.cap[g] = 0;
      L.n = n;
      if (n > 0) PG_CUDA(cudaMalloc(&L.cb, size_t(G) * n * sizeof(uint2)));
    }
    L.staged = st; // free_lists() clears it, with every array
    ensure_tiles();
    for (int g = 0; g < G; ++g)
      if (!L.idx32[g] || L.cap[g] == 0) alloc_slots(g, L.cap[g] ? L.cap[g] : 48u);
    // after any free_lists() above: the kernel always writes *hcache
    if (!L.hcache) PG_CUDA(cudaMalloc(&L.hcache, sizeof(float)));
    if (n == 0) break;
    ListOut lo{};
    for (int g = 0; g < G; ++g) {
      lo.idx32[g] = L.idx32[g];
      lo.chunks[g] = L.chunks[g];
      lo.slots[g] = L.slots[g];
      lo.cap[g] = L.cap[g];
    }
    lo.tile_info = L.tile_info;
    lo.tile_cells = L.tile_cells;
    if (st) {
      bool ok = lo.tile_info && lo.tile_cells;
      for (int g = 0; g < G; ++g) ok = ok && lo.slots[g];
      if (!ok) throw Error("staged lists: tile tables or slot arrays missing");
    }
    size_t smem = size_t(G) * (st ? 32 : 24) * kBuildNT * 4;
    lo.cb = L.cb;
    lo.maxcnt = stats_d_ + 8;
    lo.n = uint32_t(n);
    lo.G = G;
    lo.with_gf = h != nullptr ? 1 : 0;
    PG_CUDA(cudaMemsetAsync(stats_d_ + 8, 0, 8 * sizeof(uint32_t), s));
    GridView gv = view();
    float4 const *qpos = static_cast<float4 const *>(gg_[q].pos->d);
    {
      ProfScope ps(model_->prof, "nhood_lists", s);
      bool split = !st && model_->tune.v[kTuneListSplit] != 0 && n <= kSplitMaxQueries && in_grid_[q] && G <= 2;
      if (split) {
        unsigned nb2 = unsigned(div_up(n * kSplit, size_t(kSplitNT)));
        if (G == 1) k_build_lists_split<1><<<nb2, kSplitNT, 0, s>>>(gv, xsorted_, qpos, q, lo, h, L.hcache, order);
        else k_build_lists_split<2><<<nb2, kSplitNT, 0, s>>>(gv, xsorted_, qpos, q, lo, h, L.hcache, order);
      } else if (st) {
        if (G == 1) launch_build_lists<1, true>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order);
        else launch_build_lists<2, true>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order);
      } else {
        switch (G) {
        case 1: launch_build_lists<1, false>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order); break;
        case 2: launch_build_lists<2, false>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order); break;
        case 3: launch_build_lists<3, false>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order); break;
        case 4: launch_build_lists<4, false>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order); break;
        default:
          launch_build_lists<kMaxListGroups, false>(n, smem, s, gv, xsorted_, qpos, q, lo, h, L.hcache, order);
        }
      }
      count_launch();
    }
    PG_LAUNCH_CHECK();
    // one read-back: the rows' lengths, and the grid's key statistics when
    // its layout is still to be confirmed
    if (key_check_)
      PG_CUDA(cudaMemcpyAsync(stats_h_, stats_d_, 16 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    else
      PG_CUDA(cudaMemcpyAsync(stats_h_ + 8, stats_d_ + 8, 8 * sizeof(uint32_t), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    if (key_check_) {
      key_check_ = false;
      if (!same_key(key_from_stats(stats_h_), key_)) {
        // the layout changed: a new grid (read-back layout), then these lists
        key_known_ = false;
        update(s);
        build_lists(q, L, s, h, stage);
        return;
      }
    }
    bool grow = false;
    for (int g = 0; g < G; ++g)
      if (stats_h_[8 + g] > L.cap[g]) {
        alloc_slots(g, (stats_h_[8 + g] + kChunk - 1) / kChunk * kChunk + kChunk);
        grow = true;
      }
    if (!grow) {
      // rows far shorter than the capacity (e.g. after a query at a much
      // larger radius): give the storage back and build once more, so that
      // the lists do not hold the largest capacity ever needed
      bool shrink = false;
      for (int g = 0; g < G && attempt < 7; ++g) {
        uint32_t want = std::max<uint32_t>((stats_h_[8 + g] + kChunk - 1) / kChunk * kChunk + kChunk, 48u);
        if (L.cap[g] > 2 * want && L.cap[g] > 128u) {
          alloc_slots(g, want);
          shrink = true;
        }
      }
      if (!shrink) break;
    }
    list_rebuilds++;
    if (grow && attempt == 7) throw Error("neighbour lists kept overflowing their capacity");
  }
  L.epoch = epoch_;
  L.pos_versions = pos_versions();
  L.has_gf = h != nullptr;
  L.view = NbrView{};
  L.view.hcache = L.hcache;
  for (int g = 0; g < G; ++g) {
    L.view.idx32[g] = L.idx32[g];
    L.view.chunks[g] = L.chunks[g];
    L.view.cb[g] = L.cb ? L.cb + size_t(g) * n : nullptr;
    L.view.cap[g] = L.cap[g];
    L.view.slots[g] = L.staged ? L.slots[g] : nullptr;
  }
  L.view.tile_info = L.staged ? L.tile_info : nullptr;
  L.view.tile_cells = L.staged ? L.tile_cells : nullptr;
  L.view.n = uint32_t(n);
}

NbrView const &Nhood::lists(int q, cudaStream_t s, float const *h, bool stage) {
  if (!has_grid_) throw Error("Neighborhood has not been updated");
  if (q < 0 || q >= int(gg_.size())) throw Error("invalid group index");
  Lists &L = lists_[q];
  if (!gg_[q].pos) {
    // CopyNeighbors of a group without position returns nothing
    if (L.n != gg_[q].g->count || !L.cb) {
      free_lists(L);
      L.n = gg_[q].g->count;
      if (L.n) {
        PG_CUDA(cudaMalloc(&L.cb, gg_.size() * L.n * sizeof(uint2)));
        PG_CUDA(cudaMemsetAsync(L.cb, 0, gg_.size() * L.n * sizeof(uint2), s));
      }
      if (!L.hcache) {
        PG_CUDA(cudaMalloc(&L.hcache, sizeof(float)));
        float nan = std::numeric_limits<float>::quiet_NaN();
        PG_CUDA(cudaMemcpy(L.hcache, &nan, sizeof(float), cudaMemcpyHostToDevice));
      }
      L.view = NbrView{};
      for (size_t g = 0; g < gg_.size(); ++g) L.view.cb[g] = L.cb ? L.cb + g * L.n : nullptr;
      L.view.n = uint32_t(L.n);
      L.view.hcache = L.hcache;
    }
    return L.view;
  }
  // stale lists are built in the form asked for; fresh staged lists also
  // serve a caller that did not ask for staging
  if (!lists_fresh(L) || (h && !L.has_gf)) build_lists(q, L, s, h, stage);
  else if (stage && !L.staged) build_lists(q, L, s, h, true);
  return L.view;
}

// Neighborhood::Permute (util/neighborhood.cpp:106-154): per group the raw
// indices in sorted order, applied to every varying field, then Update
void Nhood::permute(Model &m, cudaStream_t s) {
  if (&m != model_) throw Error("Neighborhood::Permute with a model that was not loaded");
  if (!has_grid_) update(s);
  settle(s);
  int G = int(gg_.size());
  for (int g = 0; g < G; ++g) {
    if (!in_grid_[g] || gg_[g].g->count == 0) continue;
    size_t n = gg_[g].g->count;
    k_group_flags<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, N_, uint32_t(g), flags_); count_launch();
    PG_LAUNCH_CHECK();
    exclusive_scan(flags_, scan_, N_, block_sums_, block_sums_cap_, s);
    uint32_t *perm = nullptr;
    PG_CUDA(cudaMallocAsync(&perm, n * 4, s));
    k_group_perm<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, flags_, scan_, N_, perm); count_launch();
    PG_LAUNCH_CHECK();
    gg_[g].g->permute(perm, s);
    PG_CUDA(cudaFreeAsync(perm, s));
    permuted_count_[g] = n;
  }
  update(s);
}

void Nhood::permute_segments(Model &m, uint8_t const *due_d, cudaStream_t s) {
  if (&m != model_) throw Error("Neighborhood::Permute with a model that was not loaded");
  if (!seg_count_) throw Error("permute_segments on an unsegmented neighbourhood");
  if (!has_grid_) update(s);
  settle(s);
  int G = int(gg_.size());
  for (int g = 0; g < G; ++g) {
    if (!in_grid_[g] || gg_[g].g->count == 0) continue;
    if (g >= int(seg_.size()) || !seg_[g]) throw Error("permute_segments: group without segments");
    size_t n = gg_[g].g->count;
    k_group_flags<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, N_, uint32_t(g), flags_); count_launch();
    PG_LAUNCH_CHECK();
    exclusive_scan(flags_, scan_, N_, block_sums_, block_sums_cap_, s);
    uint32_t *perm = nullptr;
    PG_CUDA(cudaMallocAsync(&perm, n * 4, s));
    k_group_perm<<<div_up(N_, 256), 256, 0, s>>>(sorted_vals_, flags_, scan_, N_, perm); count_launch();
    k_perm_keep<<<div_up(n, 256), 256, 0, s>>>(seg_[g], due_d, n, perm); count_launch();
    PG_LAUNCH_CHECK();
    gg_[g].g->permute(perm, s);
    PG_CUDA(cudaFreeAsync(perm, s));
    permuted_count_[g] = n;
  }
  update(s);
}

void Nhood::set_segments(std::vector<uint16_t const *> const &seg, uint32_t count) {
  if (seg.size() > size_t(kMaxGroups)) throw Error("set_segments: too many groups");
  if (count > 65536) throw Error("set_segments: at most 65536 segments");
  seg_ = seg;
  seg_count_ = count;
  seg_bits_ = 0;
  while (count > 1 && (uint32_t(1) << seg_bits_) < count) ++seg_bits_;
  has_grid_ = false;
}

uint64_t Nhood::pair_count(int q, cudaStream_t s) {
  NbrView const &v = lists(q, s);
  unsigned long long *d = nullptr;
  PG_CUDA(cudaMallocAsync(&d, sizeof *d, s));
  PG_CUDA(cudaMemsetAsync(d, 0, sizeof *d, s));
  for (size_t g = 0; g < gg_.size(); ++g)
    if (v.n && v.cb[g]) {
      k_pair_count<<<div_up(v.n, 256), 256, 0, s>>>(v.cb[g], v.n, d);
      count_launch();
    }
  PG_LAUNCH_CHECK();
  unsigned long long h = 0;
  PG_CUDA(cudaMemcpyAsync(&h, d, sizeof h, cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaFreeAsync(d, s));
  PG_CUDA(cudaStreamSynchronize(s));
  return uint64_t(h);
}

size_t Nhood::staged_tiles(int q, size_t &tiles, cudaStream_t s) {
  tiles = 0;
  auto it = lists_.find(q);
  if (it == lists_.end() || !it->second.staged) return 0;
  Lists const &L = it->second;
  size_t nt = div_up(L.n, kStageTile);
  std::vector<uint2> info(nt);
  if (nt) PG_CUDA(cudaMemcpyAsync(info.data(), L.tile_info, nt * sizeof(uint2), cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  tiles = nt;
  size_t k = 0;
  for (auto const &e : info) k += e.y != kNoStage ? 1 : 0;
  return k;
}

size_t Nhood::device_bytes() const {
  // keys 2x8, values 2x4, ukeys 16, flags 4, scan 4, r2s 4, s2c 4, cell
  // start 4, adjacency 104, cell key 8, cell index 16, sorted positions 16
  size_t b = cap_ * (16 + 8 + 16 + 4 + 4 + 4 + 4 + 4 + 104 + 8 + 16 + 16);
  b += hist_cap_ * 4 + block_sums_cap_ * 4;
  for (auto const &kv : lists_) {
    Lists const &L = kv.second;
    b += L.n * gg_.size() * sizeof(uint2);
    for (size_t g = 0; g < gg_.size() && g < size_t(kMaxGroups); ++g)
      b += L.n * (size_t(L.cap[g]) * 4 + size_t(L.cap[g] / kChunk) * kChunkBytes);
  }
  return b;
}

size_t Nhood::cell_count(cudaStream_t s) {
  settle(s);
  int c = 0;
  PG_CUDA(cudaMemcpyAsync(&c, ncells_d_, sizeof(int), cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  return size_t(c);
}

void Nhood::copy_grid(uint32_t *sorted, int32_t *cell_gi, int32_t *cell_range, int32_t *cell_adj, cudaStream_t s) {
  size_t C = cell_count(s);
  if (sorted && N_) PG_CUDA(cudaMemcpyAsync(sorted, sorted_vals_, N_ * 4, cudaMemcpyDeviceToHost, s));
  std::vector<int4> gi(C);
  std::vector<int32_t> start(C + 1);
  if (C) {
    PG_CUDA(cudaMemcpyAsync(gi.data(), cell_gi_, C * 16, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaMemcpyAsync(start.data(), cell_start_, (C + 1) * 4, cudaMemcpyDeviceToHost, s));
    if (cell_adj) PG_CUDA(cudaMemcpyAsync(cell_adj, cell_adj_, C * 26 * 4, cudaMemcpyDeviceToHost, s));
  }
  PG_CUDA(cudaStreamSynchronize(s));
  for (size_t c = 0; c < C; ++c) {
    if (cell_gi) {
      cell_gi[3 * c] = gi[c].x;
      cell_gi[3 * c + 1] = gi[c].y;
      cell_gi[3 * c + 2] = gi[c].z;
    }
    if (cell_range) {
      cell_range[2 * c] = start[c];
      cell_range[2 * c + 1] = start[c + 1];
    }
  }
}

size_t Nhood::copy_neighbors(int g, size_t i, int64_t *counts, int64_t *out, size_t cap, cudaStream_t s) {
  NbrView const &v = lists(g, s);
  int G = int(gg_.size());
  if (i >= v.n) throw Error("CopyNeighbors: index out of range");
  size_t k = 0;
  for (int ng = 0; ng < G; ++ng) {
    uint2 cb{0, 0};
    PG_CUDA(cudaMemcpyAsync(&cb, v.cb[ng] + i, sizeof(uint2), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    uint32_t cn = cb.x & ~kWide;
    counts[ng] = cn;
    if (!cn) continue;
    // the item's chunks, one per chunk plane, packed on the host
    size_t nch = v.cap[ng] / kChunk;
    std::vector<unsigned char> row(nch * kChunkBytes);
    std::vector<uint32_t> e32(v.cap[ng]);
    PG_CUDA(cudaMemcpy2DAsync(row.data(), kChunkBytes, v.chunks[ng] + i * kChunkBytes, size_t(v.n) * kChunkBytes,
                              kChunkBytes, nch, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaMemcpyAsync(e32.data(), v.idx32[ng] + i * v.cap[ng], v.cap[ng] * 4, cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
    for (uint32_t slot = 0; slot < cn; ++slot) {
      if (k < cap) out[k] = nbr_host_decode(cb, row.data(), 1, 0, e32.data(), slot);
      ++k;
    }
  }
  return k;
}

void Nhood::copy_lists(int q, int ng, int64_t *offsets, uint32_t *idx, size_t cap, cudaStream_t s) {
  NbrView const &v = lists(q, s);
  size_t n = v.n;
  std::vector<uint2> cb(n);
  offsets[0] = 0;
  if (n == 0) return;
  PG_CUDA(cudaMemcpyAsync(cb.data(), v.cb[ng], n * sizeof(uint2), cudaMemcpyDeviceToHost, s));
  PG_CUDA(cudaStreamSynchronize(s));
  uint32_t used = 0; // longest row
  for (size_t i = 0; i < n; ++i) {
    offsets[i + 1] = offsets[i] + (cb[i].x & ~kWide);
    used = std::max(used, cb[i].x & ~kWide);
  }
  if (size_t(offsets[n]) > cap) throw Error("copy_lists: capacity too small");
  // only the chunk planes and the 32-bit columns that hold entries
  used = std::min(v.cap[ng], (used + kChunk - 1) / kChunk * kChunk);
  std::vector<unsigned char> ch;
  std::vector<uint32_t> e32;
  if (v.chunks[ng] && used) {
    ch.resize(size_t(used / kChunk) * kChunkBytes * n);
    e32.resize(size_t(used) * n);
    PG_CUDA(cudaMemcpyAsync(ch.data(), v.chunks[ng], ch.size(), cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaMemcpy2DAsync(e32.data(), size_t(used) * 4, v.idx32[ng], size_t(v.cap[ng]) * 4, size_t(used) * 4, n,
                              cudaMemcpyDeviceToHost, s));
    PG_CUDA(cudaStreamSynchronize(s));
  }
  for (size_t i = 0; i < n; ++i)
    for (uint32_t k = 0; k < (cb[i].x & ~kWide); ++k)
      idx[offsets[i] + k] = nbr_host_decode(cb[i], ch.data(), n, i, e32.data() + i * used, k);
}

} // namespace prtcl_gpu
