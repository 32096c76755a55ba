// Device implementations of the generated prtcl procedures on the hot path.
//
// Every procedure is one thread per particle: the thread walks its fluid
// neighbour list(s) and then its boundary neighbour list(s) sequentially, in
// the grid's traversal order, accumulating in FP32 in exactly the operation
// order of the generated C++ (the file:line cited at each kernel).  With FMA
// contraction off this reproduces the reference arithmetic per particle.
//
// Neighbour data is gathered from packed 16-byte records (position + mass,
// position + volume, position + m/rho) and the kernel gradient of a pair is
// rebuilt from the factor cached in the neighbour list; both hold values
// computed with the same operations as the on-the-fly expressions, so the
// results stay bit-identical (kernels fall back to the full kernel-gradient
// evaluation if the smoothing scale changed after the lists were built).
//
// Reductions that decide convergence (IISPH density error, PCG dot products)
// are FP64 with a fixed, batch-independent order: per-block tree sums, then
// the last block of the launch sums the block partials.  The relaxed-Jacobi
// loop (iisph.solve_pressure) and the PCG loop run on the device as CUDA
// graphs with a conditional while node: no host round trip per iteration.
#include "mat3.cuh"
#include "nbr_walk.cuh"
#include "schemes.hpp"

#include <algorithm>
#include <cstring>
#include <tuple>

namespace prtcl_gpu {

// kernels executed by device-side loops (graph bodies); read by the host
// through launch_count()
__device__ unsigned long long g_loop_kernels = 0;

namespace {

constexpr int kNT = 128;            // threads per block for particle kernels
// resident blocks per SM the neighbour sweeps are compiled for (caps their
// registers at 64): the sweeps wait on gathers, and more resident warps hide
// more of that latency
constexpr int kMinBlocks = 8;
constexpr int kMaxRedBlocks = 4096; // block partials per reduced value

// model scratch layout
constexpr int kSPcg = 0;     // scalars[0..7]: PCG
constexpr int kSJacobi = 16; // scalars[16]: FP64 density error
constexpr int kStPcgIter = 0, kStPcgActive = 1, kStPcgBody = 2;
constexpr int kStJacIter = 4, kStJacDone = 5;

// ---------------------------------------------------------------------------
// argument structs
// ---------------------------------------------------------------------------

// the pair's kernel gradient: from the cached factor (bit-identical to
// kgradW) when the lists were built with the current smoothing scale
__device__ __forceinline__ f3 pgrad(bool cached, float factor, KernelParams const &K, f3 xij) {
  return cached ? kgrad_from(factor, xij) : kgradW(K, xij);
}

struct FluidN {
  NbrList L;
  float4 const *xm; // (x, y, z, m)
  float4 const *v;  // velocity
  float4 const *a;  // acceleration
  float const *pr;  // p / (rho rho)
};

struct BoundN {
  NbrList L;
  float4 const *xV; // (x, y, z, V)
  float const *mu;  // uniform dynamic_viscosity (wkbb18)
};

template <int NF, int NB> struct Nbrs {
  FluidN f[NF > 0 ? NF : 1];
  BoundN b[NB > 0 ? NB : 1];
  float const *hcache; // smoothing scale of the cached gradient factors
};
template <class N> __device__ __forceinline__ bool use_cache(N const &nb, KernelParams const &K) {
  return *nb.hcache == K.h;
}

struct Globals {
  float const *h;
  float const *dt;
  float const *t;
  float const *fade;
  float const *omega;
  float *aprde;
  int *nprde;
  float const *gravity; // 3 floats
  float *max_speed;
  int const *jac_max;   // iisph_maximum_iterations
  float const *jac_eta; // iisph_maximum_density_error
  int *jac_iters;       // iisph_iterations
};

struct Red {
  double *partials; // [3][kMaxRedBlocks]
  unsigned *ticket;
  double *scalars;
  int *status;
  double *stats; // device-loop statistics (Model::stats_d)
};

__device__ __forceinline__ uint32_t grid_tid() { return blockIdx.x * blockDim.x + threadIdx.x; }


// FP64 block sums of NV values, committed by the last block of the launch.
// Returns true in the last block; out[] is valid in its thread 0.
template <int NV>
__device__ bool reduce_commit(double const (&v)[NV], Red const &R, double (&out)[NV]) {
  __shared__ double sh[32];
  __shared__ int last;
  for (int k = 0; k < NV; ++k) {
    double s = block_sum(v[k], sh);
    if (threadIdx.x == 0) R.partials[k * kMaxRedBlocks + blockIdx.x] = s;
  }
  __threadfence();
  if (threadIdx.x == 0) last = (atomicAdd(R.ticket, 1u) == gridDim.x - 1) ? 1 : 0;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  for (int k = 0; k < NV; ++k) {
    double acc = 0.0;
    for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x)
      acc += __ldcg(&R.partials[k * kMaxRedBlocks + b]);
    out[k] = block_sum(acc, sh);
  }
  if (threadIdx.x == 0) *R.ticket = 0u;
  return true;
}

unsigned red_grid(size_t n) { return unsigned(std::min<size_t>(div_up(n, kNT), kMaxRedBlocks)); }

// Launch shapes of the tuned sweeps (Model::tune): threads per block,
// blocks resident per SM (which caps the registers) and the neighbour-walk
// batch.  Entry 0 is the default.  Every entry computes the same bits: the
// per-item arithmetic does not depend on the shape, and the sweeps with an
// FP64 reduction keep 128 threads per block and their grid, so the shape of
// the reduction tree does not change.
template <int NT_, int MINB_, int BT_> struct Shape {
  static constexpr int nt = NT_, minb = MINB_, bt = BT_;
};
// sweeps without a reduction: the block size may change too
template <int B0, int B1>
using FreeShapes = std::tuple<Shape<kNT, kMinBlocks, B0>, Shape<kNT, kMinBlocks, B1>, Shape<256, 4, B0>,
                              Shape<512, 2, B0>>;
// sweeps with an FP64 reduction, and the tiled sweeps of a batched model
template <int B0, int B1>
using RedShapes = std::tuple<Shape<kNT, kMinBlocks, B0>, Shape<kNT, kMinBlocks, B1>, Shape<kNT, 6, B0>,
                             Shape<kNT, 12, B0>>;
// f(shape) with the knob's shape where the layout is tuned, else the default
template <class Shapes, bool Tuned, class F> void with_shape(int v, F &&f) {
  if constexpr (Tuned) {
    switch (v) {
    case 1: f(std::tuple_element_t<1, Shapes>{}); return;
    case 2: f(std::tuple_element_t<2, Shapes>{}); return;
    case 3: f(std::tuple_element_t<3, Shapes>{}); return;
    default: break;
    }
  }
  f(std::tuple_element_t<0, Shapes>{});
}
template <class Sh> std::string shape_text() {
  return std::to_string(Sh::nt) + "x" + std::to_string(Sh::minb) + "/" + std::to_string(Sh::bt);
}
template <class Shapes> std::string shapes_text() {
  return "0=" + shape_text<std::tuple_element_t<0, Shapes>>() + " 1=" + shape_text<std::tuple_element_t<1, Shapes>>() +
         " 2=" + shape_text<std::tuple_element_t<2, Shapes>>() + " 3=" + shape_text<std::tuple_element_t<3, Shapes>>();
}
using DensityShapes = FreeShapes<16, 8>;
using SetupShapes = FreeShapes<8, 16>;
using AccelShapes = FreeShapes<8, 16>;
using AccelSegShapes = RedShapes<8, 16>;
using PressureShapes = RedShapes<16, 8>;
using DiagShapes = FreeShapes<8, 16>;
using PcgShapes = RedShapes<8, 16>;

// Staged sweeps (the `staging` knob; lists built staged, nhood.hpp): a
// block's items are the tiles of kStageTile consecutive items the list build
// staged; per tile the block copies the tile's staged items' records to
// shared memory (two float4 per item, in slot order) and the threads read
// their neighbours from there by the lists' slots.  A tile that did not fit
// takes the global gathers.  The records and the order of the terms are
// those of the unstaged sweeps, so the results are bit-identical.
static_assert(kNT == int(kStageTile), "a staged sweep's block is one tile");
struct StageArgs {
  uint16_t const *fslots, *bslots; // slots of the fluid group's lists towards itself and the boundary group
  uint2 const *tile_info, *tile_cells;
  uint32_t const *sorted;          // sorted handles (group << 28 | index)
  int fg, bg;                      // the two groups' indices
};
constexpr size_t kStageSmem = 2 * kStageCap * sizeof(float4);

// copies tile `tile`'s staged records (rec(handle, x, y) per item) to sx, sy;
// false (block-uniform) for a tile that was not staged
// asynchronous global -> shared copies (cp.async): 16 bytes (L2 only), or
// 4 bytes; the records of a tile are all in flight at once
__device__ __forceinline__ void cp_async16(float4 *dst, void const *src) {
  uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async4(float *dst, void const *src) {
  uint32_t d = static_cast<uint32_t>(__cvta_generic_to_shared(dst));
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// copies tile `tile`'s staged records to sx, sy: rec(handle, sx + p, sy + p)
// issues the copies of slot p (only the parts its sweep reads); false
// (block-uniform) for a tile that was not staged
template <class Rec>
__device__ bool stage_copy(StageArgs const &SA, uint32_t tile, float4 *sx, float4 *sy, Rec &&rec) {
  __shared__ uint32_t s_src[kStageCap]; // sorted index of each staged slot
  __shared__ uint2 s_info;
  if (threadIdx.x == 0) s_info = SA.tile_info[tile];
  __syncthreads();
  uint2 info = s_info;
  if (info.y == kNoStage) return false;
  // each staged cell's slots name its sorted range
  for (uint32_t u = threadIdx.x; u < info.x; u += blockDim.x) {
    uint2 e = SA.tile_cells[size_t(tile) * kStageCells + u];
    uint32_t end = u + 1 < info.x ? SA.tile_cells[size_t(tile) * kStageCells + u + 1].y : info.y;
    for (uint32_t q = e.y; q < end; ++q) s_src[q] = e.x + (q - e.y);
  }
  __syncthreads();
  constexpr int kU = 4; // handles loaded together
  for (uint32_t p0 = threadIdx.x; p0 < info.y; p0 += kU * blockDim.x) {
    uint32_t h[kU];
#pragma unroll
    for (int k = 0; k < kU; ++k) {
      uint32_t p = p0 + k * blockDim.x;
      h[k] = p < info.y ? __ldg(SA.sorted + s_src[p]) : 0u;
    }
#pragma unroll
    for (int k = 0; k < kU; ++k) {
      uint32_t p = p0 + k * blockDim.x;
      if (p < info.y) rec(h[k], sx + p, sy + p);
    }
  }
  cp_async_wait_all();
  __syncthreads();
  return true;
}

// Batched (segmented) models: block b of a tiled launch handles tile b, up to
// kSegTile consecutive items of one slot (scene).  Reductions are per slot:
// each tile stores its FP64 block sum; the last tile of the slot to finish
// sums the slot's tile partials in tile order (one warp, fixed order), so a
// slot's sums depend only on its own items.
static_assert(kNT == int(kSegTile), "tiled kernels run one tile per block");
struct SegArgs {
  uint4 const *tiles;         // (slot, begin, end, 0)
  uint32_t const *slot_tiles; // [slots + 1]
  uint16_t const *seg;        // slot of each item
  uint32_t ntiles, slots;
  double *partials;           // [3][pcap]
  size_t pcap;
  unsigned *tickets;          // [slots]
  double *scal;               // [slots][16]
  int *stat;                  // [slots][8]
  double *stats;              // [slots][8]
  int const *nprde;           // [slots]
  int *iters;                 // [slots]
  uint32_t *active;           // tiles of the slots still iterating ([nactive[0]])
  uint32_t *nactive;          // [0] their count, [1] / [2] work counters (acceleration / pressure)
};
constexpr int kSegScal = 16, kSegStat = 8, kSegStats = 8;
// blocks of the kernels that walk the active tiles (a multiple of the SM
// count times the blocks resident per SM)
constexpr uint32_t kActiveBlocks = 152 * 8;
constexpr int kSsAprde = 8;        // scal: density error of the iteration
constexpr int kSegUpdateNT = 32;   // threads of a tiled PCG update block
constexpr int kStPcgEnded = 3;     // stat: the slot's PCG loop has ended

template <int NV>
__device__ bool seg_commit(double const (&v)[NV], SegArgs const &S, uint32_t slot, double (&out)[NV],
                           uint32_t tile) {
  __shared__ double sh[32];
  __shared__ int last;
  for (int k = 0; k < NV; ++k) {
    double s = block_sum(v[k], sh);
    if (threadIdx.x == 0) S.partials[k * S.pcap + tile] = s;
  }
  __threadfence();
  uint32_t t0 = S.slot_tiles[slot], t1 = S.slot_tiles[slot + 1];
  if (threadIdx.x == 0) last = (atomicAdd(&S.tickets[slot], 1u) == t1 - t0 - 1) ? 1 : 0;
  __syncthreads();
  if (!last) return false;
  __threadfence();
  if (threadIdx.x < 32) {
    for (int k = 0; k < NV; ++k) {
      double acc = 0.0;
      for (uint32_t t = t0 + threadIdx.x; t < t1; t += 32) acc += __ldcg(&S.partials[k * S.pcap + t]);
      out[k] = warp_sum(acc);
    }
  }
  if (threadIdx.x == 0) S.tickets[slot] = 0u;
  return true;
}

// The tiles of the slots whose Jacobi loop still iterates, in slot order
// (one block, all threads): the Jacobi sweeps of a batched model walk this
// list, so that the slots that have converged cost nothing in the
// iterations that follow.
__device__ void seg_list_active(SegArgs const &S) {
  __shared__ uint32_t warp_tot[32];
  __shared__ uint32_t base;
  if (threadIdx.x == 0) base = 0;
  __syncthreads();
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  for (uint32_t s0 = 0; s0 < S.slots; s0 += blockDim.x) {
    uint32_t sl = s0 + threadIdx.x;
    uint32_t t0 = 0, cnt = 0;
    if (sl < S.slots && !S.stat[sl * kSegStat + kStJacDone]) {
      t0 = S.slot_tiles[sl];
      cnt = S.slot_tiles[sl + 1] - t0;
    }
    // block-exclusive prefix of the counts
    uint32_t incl = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) warp_tot[w] = incl;
    __syncthreads();
    uint32_t wbase = 0, total = 0;
    for (int k = 0; k < nw; ++k) {
      if (k < w) wbase += warp_tot[k];
      total += warp_tot[k];
    }
    uint32_t off = base + wbase + incl - cnt;
    for (uint32_t j = 0; j < cnt; ++j) S.active[off + j] = t0 + j;
    __syncthreads();
    if (threadIdx.x == 0) base += total;
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    S.nactive[0] = base;
    S.nactive[1] = 0u; // the persistent sweeps of the next iteration start at tile 0
    S.nactive[2] = 0u;
  }
}
__global__ void k_seg_active(SegArgs S) { seg_list_active(S); }

// ---------------------------------------------------------------------------
// density.compute_density (schemes/density.hpp:160-220)
//   rho_i = sum_f m_j W(x_ij) + sum_b (V_j rho0) W(x_ij)
// ---------------------------------------------------------------------------

template <int NF, int NB, int NT = kNT, int MINB = kMinBlocks, int BT = 16>
__global__ void __launch_bounds__(NT, MINB) k_density(uint32_t n, float4 const *__restrict__ x, float *__restrict__ rho,
                                                 float const *rho0p, Globals G, Nbrs<NF, NB> N) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  float rho0 = *rho0p;
  f3 xi = mk3(x[i]);
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr<BT>(F.L, i, false, [&](uint32_t j_, float) {
      float4 xm = __ldg(F.xm + j_);
      acc += xm.w * kW(K, sub3(xi, mk3(xm)));
    });
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr<BT>(B.L, i, false, [&](uint32_t j_, float) {
      float4 xv = __ldg(B.xV + j_);
      acc += (xv.w * rho0) * kW(K, sub3(xi, mk3(xv)));
    });
  }
  rho[i] = acc;
}

// aiast12.compute_volume (schemes/aiast12.hpp:125-175): V_i = 1 / sum_b W
template <int NB>
__global__ void __launch_bounds__(kNT, kMinBlocks) k_volume(uint32_t n, float4 const *__restrict__ x, float *__restrict__ V,
                                                Globals G, Nbrs<0, NB> N) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  f3 xi = mk3(x[i]);
  float acc = 0.0f;
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr(B.L, i, false, [&](uint32_t j_, float) { acc += kW(K, sub3(xi, mk3(__ldg(B.xV + j_))));
    });
  }
  V[i] = 1.0f / acc;
}

// gravity.initialize_acceleration (schemes/gravity.hpp:133-158): a = g
__global__ void k_gravity(uint32_t n, float4 *__restrict__ a, Globals G) {
  uint32_t i = grid_tid();
  if (i < n) a[i] = make_float4(G.gravity[0], G.gravity[1], G.gravity[2], 0.0f);
}

// symplectic_euler.integrate_velocity_with_hard_fade
// (schemes/symplectic_euler.hpp:172-201): v += (dt a) * [0 < (t - t_b) - fade]
__global__ void k_integrate_velocity(uint32_t n, float4 *__restrict__ v, float4 const *__restrict__ a,
                                     float const *__restrict__ tb, Globals G) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  float dt = *G.dt, t = *G.t, fade = *G.fade;
  float u = ustep(0.0f, (t - tb[i]) - fade);
  float4 vi = v[i], ai = a[i];
  vi.x = vi.x + (dt * ai.x) * u;
  vi.y = vi.y + (dt * ai.y) * u;
  vi.z = vi.z + (dt * ai.z) * u;
  v[i] = vi;
}

// order-preserving map of floats to unsigned integers (for atomicMax)
__device__ __forceinline__ unsigned f2ord(float f) {
  unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float ord2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

// symplectic_euler.integrate_position (schemes/symplectic_euler.hpp:236-270):
// x += dt v; max_speed = max(max_speed, |v|) over all dynamic particles
__global__ void k_integrate_position(uint32_t n, float4 *__restrict__ x, float4 const *__restrict__ v, Globals G,
                                     unsigned *maxord) {
  uint32_t i = grid_tid();
  float sp = -INFINITY;
  if (i < n) {
    float dt = *G.dt;
    float4 xi = x[i], vi = v[i];
    xi.x = xi.x + dt * vi.x;
    xi.y = xi.y + dt * vi.y;
    xi.z = xi.z + dt * vi.z;
    x[i] = xi;
    sp = sqrtf(nsq3(mk3(vi)));
  }
  for (int o = 16; o > 0; o >>= 1) sp = fmaxf(sp, __shfl_down_sync(0xffffffffu, sp, o));
  if ((threadIdx.x & 31) == 0 && sp > -INFINITY) atomicMax(maxord, f2ord(sp));
}
__global__ void k_max_speed_begin(Globals G, unsigned *maxord) { *maxord = f2ord(*G.max_speed); }
__global__ void k_max_speed_end(Globals G, unsigned const *maxord) { *G.max_speed = ord2f(*maxord); }

// ---------------------------------------------------------------------------
// iisph.setup (schemes/iisph.hpp:188-354)
//   pass 1: c_i = -sum_f (m_j / rho_i^2) gradW - sum_b ((0.7*2) rho0 (V_j / rho_i^2)) gradW
//   pass 2: p = 0, source term s and diagonal element AA; also p / rho^2
//           (= 0) for the pressure acceleration
// ---------------------------------------------------------------------------

// Passes 1 and 2 in one sweep: pass 2 reads only the item's own c, so each
// thread computes c over its neighbours, stores it, then walks the same (now
// cached) neighbour rows again for s and AA, with the operations of the
// generated passes.
template <int NF, int NB, int NT = kNT, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(NT, MINB) k_iisph_setup(uint32_t n, float4 const *__restrict__ x,
                                                                 float4 const *__restrict__ v,
                                                                 float4 *__restrict__ cout, float const *__restrict__ m,
                                                                 float const *__restrict__ rho, float *__restrict__ p,
                                                                 float *__restrict__ pr, float *__restrict__ s,
                                                                 float *__restrict__ AA, float const *rho0p, Globals G,
                                                                 Nbrs<NF, NB> N) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *rho0p, dt = *G.dt;
  f3 xi = mk3(x[i]);
  float ri = rho[i];
  f3 c = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr<BT>(F.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xm = __ldg(F.xm + j_);
      c = sub3(c, scl3(xm.w / (ri * ri), pgrad(uc, gf_, K, sub3(xi, mk3(xm)))));
    }, true);
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      c = sub3(c, scl3(((0.7f * 2.0f) * rho0) * (xv.w / (ri * ri)), pgrad(uc, gf_, K, sub3(xi, mk3(xv)))));
    }, true);
  }
  cout[i] = make_float4(c.x, c.y, c.z, 0.0f);
  f3 vi = mk3(v[i]), ci = c;
  float mi = m[i];
  float sa = 0.0f, aa = 0.0f;
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr<BT>(F.L, i, uc, [&](uint32_t j_, float gf_) {
      uint32_t j = j_;
      float4 xm = __ldg(F.xm + j);
      f3 g = pgrad(uc, gf_, K, sub3(xi, mk3(xm)));
      float mj = xm.w;
      sa += mj * dot3(sub3(vi, mk3(__ldg(F.v + j))), g);
      aa += mj * dot3(ci, g);
      aa -= (mj * (mi / (ri * ri))) * nsq3(g);
    });
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      f3 g = pgrad(uc, gf_, K, sub3(xi, mk3(xv)));
      float w = rho0 * xv.w;
      sa += w * dot3(sub3(vi, f3{0.0f, 0.0f, 0.0f}), g);
      aa += w * dot3(ci, g);
    });
  }
  p[i] = 0.0f;
  pr[i] = 0.0f / (ri * ri);
  s[i] = (rho0 - ri) - ((dt * (rho0 / ri)) * sa);
  AA[i] = aa * ((dt * dt) * (rho0 / ri));
}

__global__ void k_set_i32(int *p, int v) { *p = v; }

// iisph.iteration_pressure_acceleration (schemes/iisph.hpp:358-423).
// `done` (device-loop mode) skips the work once the loop has converged.
template <int NF, int NB, int BT = 8>
__device__ __forceinline__ void iisph_accel_item(uint32_t i, float4 const *__restrict__ x, float const *__restrict__ p,
                                                 float const *__restrict__ rho, float4 *__restrict__ a,
                                                 KernelParams const &K, bool uc, float rho0, Nbrs<NF, NB> const &N) {
  f3 xi = mk3(x[i]);
  float pi = p[i], ri = rho[i];
  float pri = pi / (ri * ri);
  f3 acc = {0.0f, 0.0f, 0.0f};
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr<BT>(F.L, i, uc, [&](uint32_t j_, float gf_) {
      uint32_t j = j_;
      float4 xm = __ldg(F.xm + j);
      float coef = xm.w * (pri + __ldg(F.pr + j));
      acc = sub3(acc, scl3(coef, pgrad(uc, gf_, K, sub3(xi, mk3(xm)))));
    });
  }
  float bterm = (2.0f * pi) / (ri * ri);
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      float coef = ((0.7f * rho0) * xv.w) * bterm;
      acc = sub3(acc, scl3(coef, pgrad(uc, gf_, K, sub3(xi, mk3(xv)))));
    });
  }
  a[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
}
template <int NF, int NB, int NT = kNT, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(NT, MINB) k_iisph_accel(uint32_t n, float4 const *__restrict__ x, float const *__restrict__ p,
                                                     float const *__restrict__ rho, float4 *__restrict__ a,
                                                     float const *rho0p, Globals G, Nbrs<NF, NB> N, int const *done) {
  if (done && *(volatile int const *)done) return;
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  iisph_accel_item<NF, NB, BT>(i, x, p, rho, a, K, use_cache(N, K), *rho0p, N);
}
// batched models: the tiles of the slots still iterating
// (DYN: each block takes the next tile from a work counter instead of a
// static share of the tiles; the tiles' items and arithmetic are the same)
template <int NF, int NB, int MINB = kMinBlocks, int BT = 8, bool DYN = false>
__global__ void __launch_bounds__(kNT, MINB) k_iisph_accel_seg(float4 const *__restrict__ x, float const *__restrict__ p,
                                                         float const *__restrict__ rho, float4 *__restrict__ a,
                                                         float const *rho0p, Globals G, Nbrs<NF, NB> N, SegArgs S) {
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *rho0p;
  uint32_t na = S.nactive[0];
  __shared__ uint32_t next;
  for (uint32_t t = blockIdx.x;;) {
    if (DYN) {
      if (threadIdx.x == 0) next = atomicAdd(&S.nactive[1], 1u);
      __syncthreads();
      t = next;
      __syncthreads();
    }
    if (t >= na) break;
    uint4 T = S.tiles[S.active[t]];
    uint32_t i = T.y + threadIdx.x;
    if (i < T.z) iisph_accel_item<NF, NB, BT>(i, x, p, rho, a, K, uc, rho0, N);
    if (!DYN) t += gridDim.x;
  }
}

// iisph.iteration_pressure (schemes/iisph.hpp:426-516) with the FP64
// density-error reduction.  scalars[kSJacobi] accumulates aprde across the
// fluid groups of one call: `first` starts it from the global aprde (or
// from 0 in device-loop mode, where aprde := 0 precedes every iteration),
// `last_group` stores it.  Also writes p / rho^2 for the next acceleration.
struct PressureArgs {
  float4 const *x, *a;
  float const *rho, *s, *AA;
  float *p, *pr, *Ap;
  float const *rho0;
};

// the end of iteration_pressure for one item, from its neighbour sum ap:
// Ap, the new pressure (and p / rho^2); returns the density-error term
__device__ __forceinline__ double pressure_finish(uint32_t i, PressureArgs const &A, float ap, float rho0, float dt,
                                                  float omega) {
  float ri = A.rho[i];
  ap *= (dt * dt) * (rho0 / ri);
  A.Ap[i] = ap;
  float si = A.s[i], aai = A.AA[i];
  float t = A.p[i] + ((omega * (si - ap)) * rcp0(aai, 1e-9f));
  // std::max({0, t}) returns the first largest element: t only if 0 < t
  float pn = ((0.0f < t) ? t : 0.0f) * ustep(1e-9f, fabsf(aai));
  A.p[i] = pn;
  A.pr[i] = pn / (ri * ri);
  return f2d(((ap - si) / rho0) * ustep(1e-9f, pn));
}

// one item of iteration_pressure; returns its density-error term
template <int NF, int NB, int BT = 16>
__device__ __forceinline__ double iisph_pressure_item(uint32_t i, PressureArgs const &A, KernelParams const &K, bool uc,
                                                      float rho0, float dt, float omega, Nbrs<NF, NB> const &N) {
  f3 xi = mk3(A.x[i]), ai = mk3(A.a[i]);
  float ap = 0.0f;
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr<BT>(F.L, i, uc, [&](uint32_t j_, float gf_) {
      uint32_t j = j_;
      float4 xm = __ldg(F.xm + j);
      ap += xm.w * dot3(sub3(ai, mk3(__ldg(F.a + j))), pgrad(uc, gf_, K, sub3(xi, mk3(xm))));
    });
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      ap += (rho0 * xv.w) * dot3(sub3(ai, f3{0.0f, 0.0f, 0.0f}), pgrad(uc, gf_, K, sub3(xi, mk3(xv))));
    });
  }
  return pressure_finish(i, A, ap, rho0, dt, omega);
}

template <int NF, int NB, int MINB = kMinBlocks, int BT = 16>
__global__ void __launch_bounds__(kNT, MINB) k_iisph_pressure(uint32_t n, PressureArgs A, Globals G, Nbrs<NF, NB> N, Red R,
                                                        int first, int last_group, int const *done) {
  if (done && *(volatile int const *)done) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *A.rho0, dt = *G.dt, omega = *G.omega;
  double part = 0.0;
  for (uint32_t i = grid_tid(); i < n; i += gridDim.x * blockDim.x)
    part += iisph_pressure_item<NF, NB, BT>(i, A, K, uc, rho0, dt, omega, N);
  double v[1] = {part}, out[1];
  if (reduce_commit<1>(v, R, out) && threadIdx.x == 0) {
    double start = first ? (done ? 0.0 : double(*G.aprde)) : R.scalars[kSJacobi];
    double acc = start + out[0];
    R.scalars[kSJacobi] = acc;
    if (last_group) *G.aprde = float(acc);
  }
}

// iteration_pressure over the tiles of a batched model: the density error of
// each slot's iteration goes to scal[slot][kSsAprde]
// (DYN: a persistent grid whose blocks take tiles from a work counter; the
// per-tile partial sums and their per-slot commit are unchanged)
template <int NF, int NB, int MINB = kMinBlocks, int BT = 16, bool DYN = false>
__global__ void __launch_bounds__(kNT, MINB) k_iisph_pressure_seg(PressureArgs A, Globals G, Nbrs<NF, NB> N, SegArgs S) {
  // one active tile per block (the hardware's block scheduling balances the
  // tiles' uneven costs); the blocks past the active tiles exit at once
  uint32_t na = S.nactive[0];
  if (!DYN && blockIdx.x >= na) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *A.rho0, dt = *G.dt, omega = *G.omega;
  __shared__ uint32_t next;
  for (uint32_t k = blockIdx.x;;) {
    if (DYN) {
      if (threadIdx.x == 0) next = atomicAdd(&S.nactive[2], 1u);
      __syncthreads();
      k = next;
      __syncthreads();
      if (k >= na) break;
    }
    uint32_t t = S.active[k];
    uint4 T = S.tiles[t];
    uint32_t slot = T.x;
    uint32_t i = T.y + threadIdx.x;
    double part = (i < T.z) ? iisph_pressure_item<NF, NB, BT>(i, A, K, uc, rho0, dt, omega, N) : 0.0;
    double v[1] = {part}, out[1];
    if (seg_commit<1>(v, S, slot, out, t) && threadIdx.x == 0) S.scal[slot * kSegScal + kSsAprde] = out[0];
    if (!DYN) break;
  }
}

// staged relaxed-Jacobi sweeps (one fluid and one boundary group; the
// `staging` knob).  Per tile, the staged records: a fluid item's (x, m) and
// p / rho^2 (acceleration) or acceleration (pressure); a boundary item's
// (x, V).
template <int BT = 8>
__global__ void __launch_bounds__(kNT, 4) k_iisph_accel_staged(uint32_t n, float4 const *__restrict__ x,
                                                               float const *__restrict__ p,
                                                               float const *__restrict__ rho, float4 *__restrict__ a,
                                                               float const *rho0p, Globals G, Nbrs<1, 1> N,
                                                               int const *done, StageArgs SA) {
  if (done && *(volatile int const *)done) return;
  extern __shared__ float4 sm[];
  float4 *sx = sm, *sy = sm + kStageCap;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *rho0p;
  FluidN const &F = N.f[0];
  BoundN const &B = N.b[0];
  for (uint32_t tile = blockIdx.x; size_t(tile) * kNT < n; tile += gridDim.x) {
    uint32_t i = tile * kNT + threadIdx.x;
    // fluid: (x, m) and p / rho^2 (in .x); boundary: (x, V)
    bool st = stage_copy(SA, tile, sx, sy, [&](uint32_t h, float4 *dx, float4 *dy) {
      uint32_t j = h & 0x0FFFFFFFu;
      if (int(h >> 28) == SA.fg) {
        cp_async16(dx, F.xm + j);
        cp_async4(&dy->x, F.pr + j);
      } else if (int(h >> 28) == SA.bg) {
        cp_async16(dx, B.xV + j);
      }
    });
    if (i < n) {
      if (st) {
        f3 xi = mk3(x[i]);
        float pi = p[i], ri = rho[i];
        float pri = pi / (ri * ri);
        f3 acc = {0.0f, 0.0f, 0.0f};
        for_each_staged<BT>(F.L, SA.fslots, i, [&](uint32_t sl, float gf_) {
          float4 xm = sx[sl];
          float coef = xm.w * (pri + sy[sl].x);
          acc = sub3(acc, scl3(coef, pgrad(uc, gf_, K, sub3(xi, mk3(xm)))));
        });
        float bterm = (2.0f * pi) / (ri * ri);
        for_each_staged<BT>(B.L, SA.bslots, i, [&](uint32_t sl, float gf_) {
          float4 xv = sx[sl];
          float coef = ((0.7f * rho0) * xv.w) * bterm;
          acc = sub3(acc, scl3(coef, pgrad(uc, gf_, K, sub3(xi, mk3(xv)))));
        });
        a[i] = make_float4(acc.x, acc.y, acc.z, 0.0f);
      } else {
        iisph_accel_item<1, 1, BT>(i, x, p, rho, a, K, uc, rho0, N);
      }
    }
    __syncthreads(); // the next tile reuses the shared memory
  }
}

// the tiles of a block are those of k_iisph_pressure's grid-stride items,
// so the FP64 partial sums are the same
template <int BT = 8>
__global__ void __launch_bounds__(kNT, 4) k_iisph_pressure_staged(uint32_t n, PressureArgs A, Globals G,
                                                                  Nbrs<1, 1> N, Red R, int first, int last_group,
                                                                  int const *done, StageArgs SA) {
  if (done && *(volatile int const *)done) return;
  extern __shared__ float4 sm[];
  float4 *sx = sm, *sy = sm + kStageCap;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float rho0 = *A.rho0, dt = *G.dt, omega = *G.omega;
  FluidN const &F = N.f[0];
  BoundN const &B = N.b[0];
  double part = 0.0;
  for (uint32_t tile = blockIdx.x; size_t(tile) * kNT < n; tile += gridDim.x) {
    uint32_t i = tile * kNT + threadIdx.x;
    // fluid: (x, m) and the acceleration; boundary: (x, V)
    bool st = stage_copy(SA, tile, sx, sy, [&](uint32_t h, float4 *dx, float4 *dy) {
      uint32_t j = h & 0x0FFFFFFFu;
      if (int(h >> 28) == SA.fg) {
        cp_async16(dx, F.xm + j);
        cp_async16(dy, F.a + j);
      } else if (int(h >> 28) == SA.bg) {
        cp_async16(dx, B.xV + j);
      }
    });
    if (i < n) {
      if (st) {
        f3 xi = mk3(A.x[i]), ai = mk3(A.a[i]);
        float ap = 0.0f;
        for_each_staged<BT>(F.L, SA.fslots, i, [&](uint32_t sl, float gf_) {
          float4 xm = sx[sl];
          ap += xm.w * dot3(sub3(ai, mk3(sy[sl])), pgrad(uc, gf_, K, sub3(xi, mk3(xm))));
        });
        for_each_staged<BT>(B.L, SA.bslots, i, [&](uint32_t sl, float gf_) {
          float4 xv = sx[sl];
          ap += (rho0 * xv.w) * dot3(sub3(ai, f3{0.0f, 0.0f, 0.0f}), pgrad(uc, gf_, K, sub3(xi, mk3(xv))));
        });
        part += pressure_finish(i, A, ap, rho0, dt, omega);
      } else {
        part += iisph_pressure_item<1, 1, BT>(i, A, K, uc, rho0, dt, omega, N);
      }
    }
    __syncthreads();
  }
  double v[1] = {part}, out[1];
  if (reduce_commit<1>(v, R, out) && threadIdx.x == 0) {
    double start = first ? (done ? 0.0 : double(*G.aprde)) : R.scalars[kSJacobi];
    double acc = start + out[0];
    R.scalars[kSJacobi] = acc;
    if (last_group) *G.aprde = float(acc);
  }
}

// per-slot loop start: a slot without fluid items does not iterate
__global__ void k_seg_jacobi_begin(SegArgs S) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < S.slots; k += gridDim.x * blockDim.x) {
    S.stat[k * kSegStat + kStJacIter] = 0;
    S.stat[k * kSegStat + kStJacDone] = (S.nprde[k] >= 1) ? 0 : 1;
  }
}

// per-slot relaxed-Jacobi control (the rule of k_jacobi_control, per slot);
// one block; the loop continues while any slot iterates.  stats per slot:
// 0 solves, 1 iterations, 2 solves stopped at the cap, 3 largest final
// aprde / nprde, 7 final aprde / nprde of the last solve
__global__ void k_seg_jacobi_control(Globals G, SegArgs S, cudaGraphConditionalHandle h, int use_handle,
                                     int kernels, int *all_done) {
  int any = 0;
  int maxit = *G.jac_max > 0 ? *G.jac_max : 100;
  float eta = *G.jac_eta > 0.0f ? *G.jac_eta : 1e-3f;
  for (uint32_t k = threadIdx.x; k < S.slots; k += blockDim.x) {
    int *st = S.stat + k * kSegStat;
    int done = st[kStJacDone];
    if (!done) {
      int it = st[kStJacIter] + 1;
      st[kStJacIter] = it;
      double rel = S.scal[k * kSegScal + kSsAprde] / double(S.nprde[k]);
      bool converged = it >= 2 && rel < double(eta);
      if (converged || it >= maxit || it >= 100000) done = 1;
      st[kStJacDone] = done;
      if (done) {
        double *sv = S.stats + k * kSegStats;
        sv[0] += 1.0;
        sv[1] += double(it);
        if (!converged) sv[2] += 1.0;
        if (rel > sv[3]) sv[3] = rel;
        sv[7] = rel;
      }
    }
    any |= !done;
  }
  any = __syncthreads_or(any);
  if (any) seg_list_active(S);
  else if (threadIdx.x == 0) {
    // repeats of the loop body after the end sweep nothing
    S.nactive[0] = 0u;
    S.nactive[1] = 0u;
    S.nactive[2] = 0u;
  }
  if (threadIdx.x == 0) {
    *all_done = any ? 0 : 1;
    if (kernels) atomicAdd(&g_loop_kernels, (unsigned long long)kernels);
    if (use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
  }
}

// relaxed-Jacobi loop control (share/scripts/prtcl-lua.example.lua:409-420):
// at least two iterations; stop when aprde / nprde < eta or at the cap
__global__ void k_jacobi_begin(Globals G, Red R) {
  R.status[kStJacIter] = 0;
  R.status[kStJacDone] = (*G.nprde >= 1) ? 0 : 1;
  *G.jac_iters = 0;
}
__global__ void k_jacobi_control(Globals G, Red R, cudaGraphConditionalHandle h, int use_handle, int kernels) {
  int done = R.status[kStJacDone];
  if (!done) {
    int it = R.status[kStJacIter] + 1;
    R.status[kStJacIter] = it;
    int maxit = *G.jac_max > 0 ? *G.jac_max : 100;
    float eta = *G.jac_eta > 0.0f ? *G.jac_eta : 1e-3f;
    double rel = R.scalars[kSJacobi] / double(*G.nprde);
    bool converged = it >= 2 && rel < double(eta);
    if (converged || it >= maxit || it >= 100000) done = 1;
    R.status[kStJacDone] = done;
    *G.jac_iters = it;
    if (done) {
      R.stats[0] += 1.0;
      R.stats[1] += double(it);
      if (!converged) R.stats[2] += 1.0;
      if (rel > R.stats[3]) R.stats[3] = rel;
    }
  }
  // the body's kernels ran (those of a repeat after the end return at once)
  if (kernels) atomicAdd(&g_loop_kernels, (unsigned long long)kernels);
  if (use_handle) cudaGraphSetConditional(h, done ? 0u : 1u);
}

// ---------------------------------------------------------------------------
// viscosity.accumulate_acceleration (share/schemes/viscosity.prtcl:31-66,
// generated schemes/viscosity.hpp:171-240): explicit viscosity added to a.
//   a_i += ((10 (mu_i / rho_i)) (m_j / rho_j) (v_i - v_j).x_ij / (|x_ij|^2 + 0.01 h^2)) gradW
//   a_i += ((10 (mu_b / rho_i)) (rho0 V_b / rho_i) v_i.x_ib / (|x_ib|^2 + 0.01 h^2)) gradW
// over the neighbours of every fluid group, then of every boundary group.
// The fluid records are (x, m / rho) (the packed xmr records: m_j / rho_j is
// the generated code's division).
// ---------------------------------------------------------------------------

template <int NF, int NB>
__global__ void __launch_bounds__(kNT, kMinBlocks) k_viscosity(uint32_t n, float4 const *__restrict__ x,
                                                               float4 const *__restrict__ v,
                                                               float const *__restrict__ rho, float4 *__restrict__ a,
                                                               float const *rho0p, float const *mup, Globals G,
                                                               Nbrs<NF, NB> N) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float h = K.h, rho0 = *rho0p, mu = *mup;
  float hh = (0.01f * h) * h;
  f3 xi = mk3(x[i]), vi = mk3(v[i]);
  float ri = rho[i];
  f3 ai = mk3(a[i]);
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr(F.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xr = __ldg(F.xm + j_);
      f3 xij = sub3(xi, mk3(xr));
      float coef = (((10.0f * (mu / ri)) * xr.w) * dot3(sub3(vi, mk3(__ldg(F.v + j_))), xij)) / (nsq3(xij) + hh);
      ai = add3(ai, scl3(coef, pgrad(uc, gf_, K, xij)));
    });
  }
#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    float bmu = *B.mu;
    for_each_nbr(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      f3 xij = sub3(xi, mk3(xv));
      float coef = (((10.0f * (bmu / ri)) * ((rho0 * xv.w) / ri)) * dot3(sub3(vi, f3{0.0f, 0.0f, 0.0f}), xij)) /
                   (nsq3(xij) + hh);
      ai = add3(ai, scl3(coef, pgrad(uc, gf_, K, xij)));
    });
  }
  a[i] = make_float4(ai.x, ai.y, ai.z, 0.0f);
}

// ---------------------------------------------------------------------------
// WKBB18 (schemes/wkbb18.hpp)
// ---------------------------------------------------------------------------

// correction.compute_gradient_correction (share/schemes/correction.prtcl:
// 25-43, schemes/correction.hpp:162-230):
//   L_f = invert_pm(sum_{fluid neighbours} (m_j / rho_i) gradW(x_ij) (x_j - x_i)^T)
template <int NF, int NB>
__global__ void __launch_bounds__(kNT, kMinBlocks) k_correction(uint32_t n, uint32_t cap, float4 const *__restrict__ x,
                                                                float const *__restrict__ rho, float *__restrict__ L,
                                                                Globals G, Nbrs<NF, NB> N) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  f3 xi = mk3(x[i]);
  float ri = rho[i];
  M3 A;
#pragma unroll
  for (int e = 0; e < 9; ++e) A.m[e] = 0.0f;
#pragma unroll
  for (int q = 0; q < NF; ++q) {
    FluidN const &F = N.f[q];
    for_each_nbr(F.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xm = __ldg(F.xm + j_);
      f3 xj = mk3(xm);
      f3 g = pgrad(uc, gf_, K, sub3(xi, xj));
      f3 d = sub3(xj, xi);
      float sc = xm.w / ri;
      float gv[3] = {g.x, g.y, g.z}, dv[3] = {d.x, d.y, d.z};
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) A.m[3 * c + r] = A.m[3 * c + r] + sc * (gv[r] * dv[c]);
    });
  }
  M3 R = pinv3(A);
#pragma unroll
  for (int e = 0; e < 9; ++e) L[size_t(e) * cap + i] = R.m[e];
}

__global__ void k_identity9(uint32_t n, uint32_t cap, float *L) {
  uint32_t i = grid_tid();
  if (i < n)
#pragma unroll
    for (int e = 0; e < 9; ++e) L[size_t(e) * cap + i] = (e % 4 == 0) ? 1.0f : 0.0f;
}

// wkbb18.compute_diagonal (schemes/wkbb18.hpp:194-270): block-Jacobi
// preconditioner sp_i = (I - dt S_i)^-1, stored as 9 planes.  The fluid sum
// runs over the particle's own group (`foreach _ neighbor`); xmr holds
// (x, m / rho).
// GC (wkbb18_gc, share/schemes/wkbb18_gc.prtcl): every kernel gradient
// premultiplied by the item's gradient correction L_i (planar, capacity lcap)
template <int NB, bool GC = false, int NT = kNT, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(NT, MINB) k_wkbb18_diag(uint32_t n, uint32_t cap, float4 const *__restrict__ xmr,
                                                     float const *__restrict__ rho, float *__restrict__ sp,
                                                     float const *rho0p, float const *mup, Globals G, NbrList self,
                                                     Nbrs<0, NB> N, float const *__restrict__ Lc, uint32_t lcap) {
  uint32_t i = grid_tid();
  if (i >= n) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float Li[9];
  if (GC)
#pragma unroll
    for (int e = 0; e < 9; ++e) Li[e] = Lc[size_t(e) * lcap + i];
  float h = K.h, dt = *G.dt, rho0 = *rho0p, mu = *mup;
  f3 xi = mk3(xmr[i]);
  float ri = rho[i];
  float S[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) S[k] = 0.0f;
  float hh = (0.01f * h) * h;
  float cmu = 10.0f * (mu / ri);
  for_each_nbr<BT>(self, i, uc, [&](uint32_t j_, float gf_) {
    float4 xj = __ldg(xmr + j_);
    f3 xij = sub3(xi, mk3(xj));
    float coef = (cmu * xj.w) / (nsq3(xij) + hh);
    f3 g = pgrad(uc, gf_, K, xij);
    if (GC) g = mv3(Li, g);
    float gv[3] = {g.x, g.y, g.z}, xv[3] = {xij.x, xij.y, xij.z};
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) S[3 * c + r] += coef * (gv[r] * xv[c]);
    });

#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    float bmu = *B.mu;
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      f3 xij = sub3(xi, mk3(xv));
      float coef = ((10.0f * (bmu / ri)) * ((rho0 * xv.w) / ri)) / (nsq3(xij) + hh);
      f3 g = pgrad(uc, gf_, K, xij);
      if (GC) g = mv3(Li, g);
      float gv[3] = {g.x, g.y, g.z}, xw[3] = {xij.x, xij.y, xij.z};
#pragma unroll
      for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) S[3 * c + r] += coef * (gv[r] * xw[c]);
    });
  }
  M3 A;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) A.m[3 * c + r] = (r == c ? 1.0f : 0.0f) - dt * S[3 * c + r];
  M3 inv = minv3(A);
#pragma unroll
  for (int k = 0; k < 9; ++k) sp[size_t(k) * cap + i] = inv.m[k];
}

// y = sp * r  (row . vector, a0 + (a1 + a2))
__device__ __forceinline__ f3 precond(float const *__restrict__ sp, uint32_t cap, uint32_t i, f3 r) {
  float s[9];
#pragma unroll
  for (int k = 0; k < 9; ++k) s[k] = sp[size_t(k) * cap + i];
  return {s[0] * r.x + (s[3] * r.y + s[6] * r.z), s[1] * r.x + (s[4] * r.y + s[7] * r.z),
          s[2] * r.x + (s[5] * r.y + s[8] * r.z)};
}

struct PcgArgs {
  uint32_t n, cap;
  float4 const *xmr; // (x, m / rho)
  float4 const *v;
  float const *rho;
  float const *sp;
  float const *tb;
  float4 *vd;
  float4 *a;
  float4 *X, *Y, *Rr, *P, *Q;
  float const *rho0, *mu, *tol;
  int const *max_k;
  int *iterations; // uniform wkbb18_iterations
  NbrList self;
  float const *L;  // gradient correction (wkbb18_gc), planar with capacity lcap
  uint32_t lcap;
};

// system product of wkbb18.accumulate_acceleration (schemes/wkbb18.hpp:
// 339-396): (A w)_i = w_i - dt * a_f(w)_i
template <int NB, bool GC, int BT = 8>
__device__ __forceinline__ f3 wkbb18_system(PcgArgs const &P, KernelParams const &K, bool uc, float dt, float rho0,
                                            float mu, Nbrs<0, NB> const &N, float4 const *__restrict__ w, uint32_t i) {
  float Li[9];
  if (GC)
#pragma unroll
    for (int e = 0; e < 9; ++e) Li[e] = P.L[size_t(e) * P.lcap + i];
  float h = K.h;
  float hh = (0.01f * h) * h;
  f3 xi = mk3(P.xmr[i]), wi = mk3(w[i]);
  float ri = P.rho[i];
  float cmu = 10.0f * (mu / ri);
  f3 af = {0.0f, 0.0f, 0.0f};
  for_each_nbr<BT>(P.self, i, uc, [&](uint32_t j_, float gf_) {
    uint32_t j = j_;
    float4 xj = __ldg(P.xmr + j);
    f3 xij = sub3(xi, mk3(xj));
    float coef = ((cmu * xj.w) * dot3(sub3(wi, mk3(__ldg(w + j))), xij)) / (nsq3(xij) + hh);
    f3 g = pgrad(uc, gf_, K, xij);
    if (GC) g = mv3(Li, g);
    af = add3(af, scl3(coef, g));
    });

#pragma unroll
  for (int q = 0; q < NB; ++q) {
    BoundN const &B = N.b[q];
    float bmu = *B.mu;
    float cb_mu = 10.0f * (bmu / ri);
    for_each_nbr<BT>(B.L, i, uc, [&](uint32_t j_, float gf_) {
      float4 xv = __ldg(B.xV + j_);
      f3 xij = sub3(xi, mk3(xv));
      float coef = ((cb_mu * ((rho0 * xv.w) / ri)) * dot3(wi, xij)) / (nsq3(xij) + hh);
      f3 g = pgrad(uc, gf_, K, xij);
      if (GC) g = mv3(Li, g);
      af = add3(af, scl3(coef, g));
    });
  }
  return sub3(wi, scl3(dt, af));
}

// scalars: 0 b_nsq, 1 thr, 2 r_nsq, 3 next_rdy, 4 prev_rdy, 5 pdq,
// 6 alpha, 7 beta (f32 values held in double slots)
__global__ void k_pcg_guess(PcgArgs P) {
  uint32_t i = grid_tid();
  if (i < P.n) P.X[i] = P.v[i];
}

__device__ __forceinline__ void pcg_init_finish(PcgArgs const &P, uint32_t i, f3 ax, double &bb, double &rr,
                                                double &ry);
// the rest of pcg_q_item from q = A p: stores q, returns p . q
__device__ __forceinline__ double pcg_q_finish(PcgArgs const &P, uint32_t i, f3 q) {
  P.Q[i] = make_float4(q.x, q.y, q.z, 0.0f);
  return f2d(dot3(mk3(P.P[i]), q));
}

// r = A x - b (b = v: the right-hand side's boundary term has v_b = 0),
// y = M r, p = -y; dots b.b, r.r, r.y (solver/cg_openmp.hpp:48-96)
// per-item parts of the PCG kernels (shared by the plain and the tiled
// launches, so both compute the same values)
template <int NB, bool GC, int BT = 8>
__device__ __forceinline__ void pcg_init_item(PcgArgs const &P, KernelParams const &K, bool uc, float dt, float rho0,
                                              float mu, Nbrs<0, NB> const &N, uint32_t i, double &bb, double &rr,
                                              double &ry) {
  pcg_init_finish(P, i, wkbb18_system<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, P.X, i), bb, rr, ry);
}
// the rest of pcg_init_item from A x
__device__ __forceinline__ void pcg_init_finish(PcgArgs const &P, uint32_t i, f3 ax, double &bb, double &rr,
                                                double &ry) {
  f3 b = mk3(P.v[i]);
  f3 r = sub3(ax, b);
  f3 y = precond(P.sp, P.cap, i, r);
  P.Rr[i] = make_float4(r.x, r.y, r.z, 0.0f);
  P.Y[i] = make_float4(y.x, y.y, y.z, 0.0f);
  P.P[i] = make_float4(-y.x, -y.y, -y.z, 0.0f);
  bb += f2d(dot3(b, b));
  rr += f2d(dot3(r, r));
  ry += f2d(dot3(r, y));
}
template <int NB, bool GC, int BT = 8>
__device__ __forceinline__ double pcg_q_item(PcgArgs const &P, KernelParams const &K, bool uc, float dt, float rho0,
                                             float mu, Nbrs<0, NB> const &N, uint32_t i) {
  return pcg_q_finish(P, i, wkbb18_system<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, P.P, i));
}
__device__ __forceinline__ void pcg_update_item(PcgArgs const &P, float alpha, uint32_t i, double &rr, double &ry) {
  f3 x = mk3(P.X[i]), p = mk3(P.P[i]), r = mk3(P.Rr[i]), q = mk3(P.Q[i]);
  x = add3(x, scl3(alpha, p));
  r = add3(r, scl3(alpha, q));
  f3 y = precond(P.sp, P.cap, i, r);
  P.X[i] = make_float4(x.x, x.y, x.z, 0.0f);
  P.Rr[i] = make_float4(r.x, r.y, r.z, 0.0f);
  P.Y[i] = make_float4(y.x, y.y, y.z, 0.0f);
  rr += f2d(dot3(r, r));
  ry += f2d(dot3(r, y));
}
__device__ __forceinline__ void pcg_p_item(PcgArgs const &P, float beta, uint32_t i) {
  f3 y = mk3(P.Y[i]), p = mk3(P.P[i]);
  f3 r = add3(f3{-y.x, -y.y, -y.z}, scl3(beta, p));
  P.P[i] = make_float4(r.x, r.y, r.z, 0.0f);
}
// solver scalars after the initial residual (thr = max(tol^2 |b|^2, FLT_MIN))
__device__ __forceinline__ void pcg_init_scalars(double *sc, int *st, double const (&out)[3], float tol_f) {
  double tol = double(tol_f);
  sc[0] = out[0];
  double thr = tol * tol * out[0], fmin_ = double(1.17549435082228750797e-38f);
  sc[1] = (thr < fmin_) ? fmin_ : thr;
  sc[2] = out[1];
  sc[3] = out[2];
  st[kStPcgIter] = 0;
  st[kStPcgActive] = 1; // iteration 0 always runs (min_k = 1)
  st[kStPcgBody] = 0;
}
// after p.q: alpha, or stop on |p.q| < tol
__device__ __forceinline__ void pcg_q_scalars(double *sc, int *st, double pq, float tol) {
  double prev = sc[3];
  sc[4] = prev;
  sc[5] = pq;
  if (fabs(pq) < double(tol)) st[kStPcgActive] = 0;
  else sc[6] = double(float(prev / pq));
}
// after the update: stop on |r.y| < tol, else beta, k + 1 and the loop test
__device__ __forceinline__ void pcg_update_scalars(double *sc, int *st, double rr, double ry, float tol, int max_k) {
  double prev = sc[4];
  sc[2] = rr;
  sc[3] = ry;
  if (fabs(prev) < double(tol)) {
    st[kStPcgActive] = 0;
  } else {
    sc[7] = double(float(ry / prev));
    int k = st[kStPcgIter] + 1;
    st[kStPcgIter] = k;
    // loop condition ok(k, r_nsq): k < 1 -> run; k > max_k -> stop;
    // r_nsq < thr -> stop
    bool ok = (k < 1) || (!(k > max_k) && !(rr < sc[1]));
    st[kStPcgActive] = ok ? 1 : 0;
  }
}

template <int NB, bool GC = false, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(kNT, MINB) k_pcg_init(PcgArgs P, Globals G, Nbrs<0, NB> N, Red R) {
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  double bb = 0.0, rr = 0.0, ry = 0.0;
  for (uint32_t i = grid_tid(); i < P.n; i += gridDim.x * blockDim.x)
    pcg_init_item<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, i, bb, rr, ry);
  double v[3] = {bb, rr, ry}, out[3];
  if (reduce_commit<3>(v, R, out) && threadIdx.x == 0) pcg_init_scalars(R.scalars + kSPcg, R.status, out, *P.tol);
}

// q = A p; p.q; alpha or break (solver/cg_openmp.hpp:121-151)
template <int NB, bool GC = false, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(kNT, MINB) k_pcg_q(PcgArgs P, Globals G, Nbrs<0, NB> N, Red R) {
  if (!*(volatile int *)&R.status[kStPcgActive]) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  double pq = 0.0;
  for (uint32_t i = grid_tid(); i < P.n; i += gridDim.x * blockDim.x)
    pq += pcg_q_item<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, i);
  double v[1] = {pq}, out[1];
  if (reduce_commit<1>(v, R, out) && threadIdx.x == 0) pcg_q_scalars(R.scalars + kSPcg, R.status, out[0], *P.tol);
}

// the system product from staged lists (one boundary group, no gradient
// correction): the staged records are a fluid item's (x, m / rho) and w, a
// boundary item's (x, V); terms and order those of wkbb18_system
template <int BT = 8>
__device__ __forceinline__ f3 wkbb18_system_staged(PcgArgs const &P, KernelParams const &K, bool uc, float dt,
                                                   float rho0, float mu, float bmu, StageArgs const &SA,
                                                   BoundN const &B, float4 const *sx, float4 const *sy,
                                                   float4 const *__restrict__ w, uint32_t i) {
  float h = K.h;
  float hh = (0.01f * h) * h;
  f3 xi = mk3(P.xmr[i]), wi = mk3(w[i]);
  float ri = P.rho[i];
  float cmu = 10.0f * (mu / ri);
  f3 af = {0.0f, 0.0f, 0.0f};
  for_each_staged<BT>(P.self, SA.fslots, i, [&](uint32_t sl, float gf_) {
    float4 xj = sx[sl];
    f3 xij = sub3(xi, mk3(xj));
    float coef = ((cmu * xj.w) * dot3(sub3(wi, mk3(sy[sl])), xij)) / (nsq3(xij) + hh);
    af = add3(af, scl3(coef, pgrad(uc, gf_, K, xij)));
  });
  float cb_mu = 10.0f * (bmu / ri);
  for_each_staged<BT>(B.L, SA.bslots, i, [&](uint32_t sl, float gf_) {
    float4 xv = sx[sl];
    f3 xij = sub3(xi, mk3(xv));
    float coef = ((cb_mu * ((rho0 * xv.w) / ri)) * dot3(wi, xij)) / (nsq3(xij) + hh);
    af = add3(af, scl3(coef, pgrad(uc, gf_, K, xij)));
  });
  return sub3(wi, scl3(dt, af));
}

// stages tile `tile` for the system product with vector w
__device__ __forceinline__ bool stage_system(StageArgs const &SA, uint32_t tile, float4 *sx, float4 *sy,
                                             PcgArgs const &P, BoundN const &B, float4 const *w) {
  // fluid: (x, m / rho) and w; boundary: (x, V)
  return stage_copy(SA, tile, sx, sy, [&](uint32_t h, float4 *dx, float4 *dy) {
    uint32_t j = h & 0x0FFFFFFFu;
    if (int(h >> 28) == SA.fg) {
      cp_async16(dx, P.xmr + j);
      cp_async16(dy, w + j);
    } else if (int(h >> 28) == SA.bg) {
      cp_async16(dx, B.xV + j);
    }
  });
}

// staged k_pcg_init / k_pcg_q (the `staging` knob): a block's tiles are the
// items of the plain kernels' grid-stride loop, so the FP64 sums are the same
template <int BT = 8>
__global__ void __launch_bounds__(kNT, 4) k_pcg_init_staged(PcgArgs P, Globals G, Nbrs<0, 1> N, Red R, StageArgs SA) {
  extern __shared__ float4 sm[];
  float4 *sx = sm, *sy = sm + kStageCap;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  BoundN const &B = N.b[0];
  float bmu = *B.mu;
  double bb = 0.0, rr = 0.0, ry = 0.0;
  for (uint32_t tile = blockIdx.x; size_t(tile) * kNT < P.n; tile += gridDim.x) {
    uint32_t i = tile * kNT + threadIdx.x;
    bool st = stage_system(SA, tile, sx, sy, P, B, P.X);
    if (i < P.n) {
      if (st)
        pcg_init_finish(P, i, wkbb18_system_staged<BT>(P, K, uc, dt, rho0, mu, bmu, SA, B, sx, sy, P.X, i), bb, rr,
                        ry);
      else
        pcg_init_item<1, false, BT>(P, K, uc, dt, rho0, mu, N, i, bb, rr, ry);
    }
    __syncthreads();
  }
  double v[3] = {bb, rr, ry}, out[3];
  if (reduce_commit<3>(v, R, out) && threadIdx.x == 0) pcg_init_scalars(R.scalars + kSPcg, R.status, out, *P.tol);
}

template <int BT = 8>
__global__ void __launch_bounds__(kNT, 4) k_pcg_q_staged(PcgArgs P, Globals G, Nbrs<0, 1> N, Red R, StageArgs SA) {
  if (!*(volatile int *)&R.status[kStPcgActive]) return;
  extern __shared__ float4 sm[];
  float4 *sx = sm, *sy = sm + kStageCap;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  BoundN const &B = N.b[0];
  float bmu = *B.mu;
  double pq = 0.0;
  for (uint32_t tile = blockIdx.x; size_t(tile) * kNT < P.n; tile += gridDim.x) {
    uint32_t i = tile * kNT + threadIdx.x;
    bool st = stage_system(SA, tile, sx, sy, P, B, P.P);
    if (i < P.n)
      pq += st ? pcg_q_finish(P, i, wkbb18_system_staged<BT>(P, K, uc, dt, rho0, mu, bmu, SA, B, sx, sy, P.P, i))
               : pcg_q_item<1, false, BT>(P, K, uc, dt, rho0, mu, N, i);
    __syncthreads();
  }
  double v[1] = {pq}, out[1];
  if (reduce_commit<1>(v, R, out) && threadIdx.x == 0) pcg_q_scalars(R.scalars + kSPcg, R.status, out[0], *P.tol);
}

// q = A p as a cell-tile sweep (the pcg_q knob's shape 4): no neighbour
// lists.  A block stages, per tile of 128 consecutive fluid items, the
// packed records of every cell adjacent to the tile's cells in shared
// memory (position and handle; the search direction and m / rho for a fluid
// item, the volume for a boundary item), and each thread walks its 27 cells
// in the lists' traversal order (own cell, adjacency slots 0..25, sorted
// order within a cell), fluid items first, then boundary items, testing
// every candidate with the exact d^2 < T of the list build and computing the
// gradient factor with the same operations.  The terms and their order are
// those of wkbb18_system, so q is bit-identical; the grid and the
// item-to-thread mapping are those of k_pcg_q, so the FP64 sum of p . q is
// too.  A tile whose cells hold more than kTileStage items (or more than
// kTileHash cells) takes the list walk instead.
constexpr int kTileStage = 1536; // staged items per tile (2 x 16 bytes each)
constexpr int kTileHash = 512;   // cells per tile (open-addressing table)

__device__ __forceinline__ uint32_t tile_hash(int c) { return (uint32_t(c) * 2654435761u) >> 23; } // 9 bits

// slot of cell c in the tile's table (the cell is present)
__device__ __forceinline__ int tile_find(int const *hkey, int c) {
  uint32_t h = tile_hash(c);
  for (int probe = 0; probe < kTileHash; ++probe) {
    int slot = int((h + uint32_t(probe)) & (kTileHash - 1));
    if (hkey[slot] == c) return slot;
  }
  return -1;
}

template <int NB>
__global__ void __launch_bounds__(kNT, 4) k_pcg_q_tiles(PcgArgs P, Globals G, Nbrs<0, NB> N, Red R, GridView gv,
                                                         float4 const *__restrict__ xs, int fg, int bg) {
  static_assert(NB == 1, "the cell-tile sweep handles one boundary group");
  if (!*(volatile int *)&R.status[kStPcgActive]) return;
  extern __shared__ float4 stage[]; // [kTileStage] records, then [kTileStage] payloads
  __shared__ int hkey[kTileHash];
  __shared__ uint32_t hval[kTileHash]; // base << 16 | count
  __shared__ int homes[kNT];
  __shared__ uint32_t wsum[kNT / 32], wocc[kNT / 32];
  __shared__ int ccell[kTileHash];     // occupied slots' cells, compacted
  __shared__ uint32_t cbase[kTileHash]; // and their staged bases (ascending)
  __shared__ int s_over, s_cells;
  float4 *pay = stage + kTileStage;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  float hh = (0.01f * K.h) * K.h;
  BoundN const &B = N.b[0];
  float bmu = *B.mu;
  double pq = 0.0;
  for (uint32_t tile = blockIdx.x; size_t(tile) * kNT < P.n; tile += gridDim.x) {
    uint32_t i = tile * kNT + threadIdx.x;
    bool has = i < P.n;
    for (int sl = threadIdx.x; sl < kTileHash; sl += kNT) {
      hkey[sl] = -1;
      hval[sl] = 0u;
    }
    if (threadIdx.x == 0) s_over = 0;
    int home = has ? gv.s2c[gv.r2s[gv.goff[fg] + i]] : -1;
    homes[threadIdx.x] = home;
    __syncthreads();
    // the first item of each run of equal home cells enters the run's 27 cells
    if (has && (threadIdx.x == 0 || homes[threadIdx.x - 1] != home)) {
      for (int k = -1; k < 26; ++k) {
        int c = k < 0 ? home : gv.cell_adj[size_t(home) * 26 + k];
        if (c < 0) continue;
        uint32_t h = tile_hash(c);
        bool placed = false;
        for (int probe = 0; probe < kTileHash && !placed; ++probe) {
          int slot = int((h + uint32_t(probe)) & (kTileHash - 1));
          int old = atomicCAS(&hkey[slot], -1, c);
          placed = old == -1 || old == c;
        }
        if (!placed) s_over = 1;
      }
    }
    __syncthreads();
    // staged ranges: each thread owns table slots tid, tid + 128, ...
    uint32_t cnt[kTileHash / kNT], mine = 0;
#pragma unroll
    for (int m = 0; m < kTileHash / kNT; ++m) {
      int c = hkey[threadIdx.x + m * kNT];
      cnt[m] = c >= 0 ? uint32_t(gv.cell_start[c + 1] - gv.cell_start[c]) : 0u;
      mine += cnt[m];
    }
    // block-exclusive prefix of the per-thread counts
    uint32_t incl = mine;
    int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      uint32_t v = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += v;
    }
    if (lane == 31) wsum[w] = incl;
    __syncthreads();
    uint32_t off = incl - mine, total = 0;
    for (int k = 0; k < kNT / 32; ++k) {
      if (k < w) off += wsum[k];
      total += wsum[k];
    }
    if (total > uint32_t(kTileStage)) s_over = 1;
    __syncthreads();
    bool over = s_over != 0;
    if (!over) {
      // bases in (thread, m) order, and the occupied slots compacted in the
      // same order, so that the compacted bases ascend
      uint32_t occ = 0;
#pragma unroll
      for (int m = 0; m < kTileHash / kNT; ++m) occ += hkey[threadIdx.x + m * kNT] >= 0 ? 1u : 0u;
      uint32_t oincl = occ;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        uint32_t v = __shfl_up_sync(0xffffffffu, oincl, o);
        if (lane >= o) oincl += v;
      }
      if (lane == 31) wocc[w] = oincl;
      __syncthreads();
      uint32_t u = oincl - occ;
      for (int k = 0; k < w; ++k) u += wocc[k];
#pragma unroll
      for (int m = 0; m < kTileHash / kNT; ++m) {
        int sl = threadIdx.x + m * kNT;
        int c = hkey[sl];
        if (c >= 0) {
          hval[sl] = (off << 16) | cnt[m];
          ccell[u] = c;
          cbase[u] = off;
          off += cnt[m];
          ++u;
        }
      }
      if (threadIdx.x == kNT - 1) s_cells = u;
    }
    __syncthreads();
    if (!over) {
      // every thread copies staged items p = tid, tid + 128, ...: the cell of
      // p is the last compacted cell whose base is <= p
      int ncel = s_cells;
      for (uint32_t pidx = threadIdx.x; pidx < total; pidx += kNT) {
        int lo = 0, hi = ncel - 1;
        while (lo < hi) {
          int mid = (lo + hi + 1) >> 1;
          if (cbase[mid] <= pidx) lo = mid;
          else hi = mid - 1;
        }
        int c = ccell[lo];
        uint32_t e = pidx - cbase[lo];
        float4 X = xs[gv.cell_start[c] + int(e)];
        uint32_t hd = __float_as_uint(X.w);
        int g = int(hd >> 28);
        uint32_t j = hd & 0x0FFFFFFFu;
        float4 W = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        if (g == fg) {
          float4 pj = P.P[j];
          W = make_float4(pj.x, pj.y, pj.z, P.xmr[j].w);
        } else if (g == bg) {
          W.w = B.xV[j].w;
        }
        stage[pidx] = X;
        pay[pidx] = W;
      }
    }
    __syncthreads();
    if (has) {
      f3 q;
      if (over) {
        q = wkbb18_system<NB, false, 8>(P, K, uc, dt, rho0, mu, N, P.P, i);
      } else {
        f3 xi = mk3(P.xmr[i]), wi = mk3(P.P[i]);
        float ri = P.rho[i];
        float cmu = 10.0f * (mu / ri);
        float cb_mu = 10.0f * (bmu / ri);
        f3 af = {0.0f, 0.0f, 0.0f};
        // fluid neighbours (the group's own lists), then boundary neighbours
        for (int pass = 0; pass < 2; ++pass) {
          int want = pass == 0 ? fg : bg;
          for (int k = -1; k < 26; ++k) {
            int c = k < 0 ? home : gv.cell_adj[size_t(home) * 26 + k];
            if (c < 0) continue;
            int sl = tile_find(hkey, c); // present: the run's first item entered it
            uint32_t hv = sl >= 0 ? hval[sl] : 0u;
            uint32_t b0 = hv >> 16, b1 = b0 + (hv & 0xFFFFu);
            for (uint32_t e = b0; e < b1; ++e) {
              float4 X = stage[e];
              if (int(__float_as_uint(X.w) >> 28) != want) continue;
              f3 xij = sub3(xi, mk3(X));
              float d2 = nsq3(xij);
              if (!(d2 < gv.r2lt)) continue;
              float4 W = pay[e];
              f3 g = kgrad_from(kgrad_factor(K, d2), xij);
              float coef;
              if (pass == 0) coef = ((cmu * W.w) * dot3(sub3(wi, mk3(W)), xij)) / (nsq3(xij) + hh);
              else coef = ((cb_mu * ((rho0 * W.w) / ri)) * dot3(wi, xij)) / (nsq3(xij) + hh);
              af = add3(af, scl3(coef, g));
            }
          }
        }
        q = sub3(wi, scl3(dt, af));
      }
      P.Q[i] = make_float4(q.x, q.y, q.z, 0.0f);
      pq += f2d(dot3(mk3(P.P[i]), q));
    }
    __syncthreads(); // the next tile reuses the shared memory
  }
  double v[1] = {pq}, out[1];
  if (reduce_commit<1>(v, R, out) && threadIdx.x == 0) pcg_q_scalars(R.scalars + kSPcg, R.status, out[0], *P.tol);
}

// x += alpha p; r += alpha q; y = M r; r.r; r.y; break / beta
// (solver/cg_openmp.hpp:153-191)
__global__ void __launch_bounds__(kNT, kMinBlocks) k_pcg_update(PcgArgs P, Red R) {
  if (!*(volatile int *)&R.status[kStPcgActive]) return;
  float alpha = float(R.scalars[kSPcg + 6]);
  double rr = 0.0, ry = 0.0;
  for (uint32_t i = grid_tid(); i < P.n; i += gridDim.x * blockDim.x) pcg_update_item(P, alpha, i, rr, ry);
  double v[2] = {rr, ry}, out[2];
  if (reduce_commit<2>(v, R, out) && threadIdx.x == 0)
    pcg_update_scalars(R.scalars + kSPcg, R.status, out[0], out[1], *P.tol, *P.max_k);
}

// p = -y + beta p (only when the loop continues)
__global__ void k_pcg_p(PcgArgs P, Red R) {
  if (!*(volatile int *)&R.status[kStPcgActive]) return;
  float beta = float(R.scalars[kSPcg + 7]);
  for (uint32_t i = grid_tid(); i < P.n; i += gridDim.x * blockDim.x) pcg_p_item(P, beta, i);
}

// loop control of the device PCG loop: continue while active, and never run
// more than max_k + 1 bodies
__global__ void k_pcg_control(PcgArgs P, Red R, cudaGraphConditionalHandle h, int use_handle, int kernels) {
  int body = R.status[kStPcgBody] + 1;
  R.status[kStPcgBody] = body;
  if (kernels) atomicAdd(&g_loop_kernels, (unsigned long long)kernels);
  int maxk = *P.max_k;
  bool cont = R.status[kStPcgActive] && body < (maxk < 0 ? 0 : maxk) + 1 && body < 1000000;
  if (!cont) {
    R.stats[4] += 1.0;
    R.stats[5] += double(R.status[kStPcgIter]);
    if (R.status[kStPcgActive]) R.stats[6] += 1.0;
    R.status[kStPcgActive] = 0;
  }
  if (use_handle) cudaGraphSetConditional(h, cont ? 1u : 0u);
}

// --- the PCG loop over the tiles of a batched model, per slot -------------

template <int NB, bool GC = false, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(kNT, MINB) k_pcg_init_seg(PcgArgs P, Globals G, Nbrs<0, NB> N, SegArgs S) {
  uint4 T = S.tiles[blockIdx.x];
  uint32_t slot = T.x;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  double bb = 0.0, rr = 0.0, ry = 0.0;
  uint32_t i = T.y + threadIdx.x;
  if (i < T.z) pcg_init_item<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, i, bb, rr, ry);
  double v[3] = {bb, rr, ry}, out[3];
  if (seg_commit<3>(v, S, slot, out, blockIdx.x) && threadIdx.x == 0) {
    int *st = S.stat + slot * kSegStat;
    pcg_init_scalars(S.scal + slot * kSegScal, st, out, *P.tol);
    st[kStPcgEnded] = 0;
  }
}

template <int NB, bool GC = false, int MINB = kMinBlocks, int BT = 8>
__global__ void __launch_bounds__(kNT, MINB) k_pcg_q_seg(PcgArgs P, Globals G, Nbrs<0, NB> N, SegArgs S) {
  uint4 T = S.tiles[blockIdx.x];
  uint32_t slot = T.x;
  if (!S.stat[slot * kSegStat + kStPcgActive]) return;
  KernelParams K = kparams(*G.h);
  bool uc = use_cache(N, K);
  float dt = *G.dt, rho0 = *P.rho0, mu = *P.mu;
  uint32_t i = T.y + threadIdx.x;
  double v[1] = {(i < T.z) ? pcg_q_item<NB, GC, BT>(P, K, uc, dt, rho0, mu, N, i) : 0.0}, out[1];
  if (seg_commit<1>(v, S, slot, out, blockIdx.x) && threadIdx.x == 0)
    pcg_q_scalars(S.scal + slot * kSegScal, S.stat + slot * kSegStat, out[0], *P.tol);
}

__global__ void __launch_bounds__(kNT, kMinBlocks) k_pcg_update_seg(PcgArgs P, SegArgs S) {
  uint4 T = S.tiles[blockIdx.x];
  uint32_t slot = T.x;
  if (!S.stat[slot * kSegStat + kStPcgActive]) return;
  float alpha = float(S.scal[slot * kSegScal + 6]);
  double rr = 0.0, ry = 0.0;
  // one warp per tile (kSegUpdateNT): each lane folds four items before the
  // FP64 tree, which this GPU's narrow FP64 pipe makes the costly part
  for (uint32_t i = T.y + threadIdx.x; i < T.z; i += blockDim.x) pcg_update_item(P, alpha, i, rr, ry);
  double v[2] = {rr, ry}, out[2];
  if (seg_commit<2>(v, S, slot, out, blockIdx.x) && threadIdx.x == 0)
    pcg_update_scalars(S.scal + slot * kSegScal, S.stat + slot * kSegStat, out[0], out[1], *P.tol, *P.max_k);
}

__global__ void k_pcg_p_seg(PcgArgs P, SegArgs S) {
  uint32_t i = grid_tid();
  if (i >= P.n) return;
  uint32_t slot = S.seg[i];
  if (!S.stat[slot * kSegStat + kStPcgActive]) return;
  pcg_p_item(P, float(S.scal[slot * kSegScal + 7]), i);
}

// per-slot PCG loop control (the rule of k_pcg_control, per slot); one
// block.  stats per slot: 4 solves, 5 iterations, 6 solves stopped by the
// iteration limit
__global__ void k_seg_pcg_control(PcgArgs P, SegArgs S, cudaGraphConditionalHandle h, int use_handle, int kernels,
                                  int *any_active) {
  int any = 0;
  int maxk = *P.max_k;
  for (uint32_t k = threadIdx.x; k < S.slots; k += blockDim.x) {
    int *st = S.stat + k * kSegStat;
    if (st[kStPcgEnded]) continue;
    int body = st[kStPcgBody] + 1;
    st[kStPcgBody] = body;
    bool cont = st[kStPcgActive] && body < (maxk < 0 ? 0 : maxk) + 1 && body < 1000000;
    if (!cont) {
      double *sv = S.stats + k * kSegStats;
      sv[4] += 1.0;
      sv[5] += double(st[kStPcgIter]);
      if (st[kStPcgActive]) sv[6] += 1.0;
      st[kStPcgActive] = 0;
      st[kStPcgEnded] = 1;
      S.iters[k] = st[kStPcgIter];
    }
    any |= cont ? 1 : 0;
  }
  any = __syncthreads_or(any);
  if (threadIdx.x == 0) {
    *any_active = any;
    if (kernels) atomicAdd(&g_loop_kernels, (unsigned long long)kernels);
    if (use_handle) cudaGraphSetConditional(h, any ? 1u : 0u);
  }
}

// slots without fluid items take no part in the loop
__global__ void k_seg_pcg_begin(SegArgs S) {
  for (uint32_t k = blockIdx.x * blockDim.x + threadIdx.x; k < S.slots; k += gridDim.x * blockDim.x) {
    int *st = S.stat + k * kSegStat;
    if (S.slot_tiles[k] == S.slot_tiles[k + 1]) {
      st[kStPcgActive] = 0;
      st[kStPcgEnded] = 1;
      st[kStPcgIter] = 0;
      S.iters[k] = 0;
    }
  }
}

// apply (schemes/wkbb18.hpp:401-413): vd = (x - v) [0 < (t - t_b) - fade];
// a = vd / dt
__global__ void k_pcg_apply(PcgArgs P, Globals G, Red R) {
  uint32_t i = grid_tid();
  if (i == 0 && R.status) *P.iterations = R.status[kStPcgIter];
  if (i >= P.n) return;
  float dt = *G.dt, t = *G.t, fade = *G.fade;
  float u = ustep(0.0f, (t - P.tb[i]) - fade);
  f3 d = scl3(u, sub3(mk3(P.X[i]), mk3(P.v[i])));
  P.vd[i] = make_float4(d.x, d.y, d.z, 0.0f);
  P.a[i] = make_float4(d.x / dt, d.y / dt, d.z / dt, 0.0f);
}

// ---------------------------------------------------------------------------
// host helpers
// ---------------------------------------------------------------------------

FieldType ft_real() { return FieldType{}; }
FieldType ft_vec3() {
  FieldType t;
  t.rank = 1;
  t.ext[0] = 3;
  return t;
}
FieldType ft_mat3() {
  FieldType t;
  t.rank = 2;
  t.ext[0] = 3;
  t.ext[1] = 3;
  return t;
}
FieldType ft_int() {
  FieldType t;
  t.ctype = CType::I32;
  return t;
}

template <class T> T *dptr(VaryingField *f) { return static_cast<T *>(f->d); }

// dispatch on the number of fluid (1..2) and boundary (0..2) neighbour groups
template <template <int, int> class F, class... A> void dispatch_fb(int nf, int nb, A &&...a) {
  if (nf == 1 && nb == 1) return F<1, 1>::go(a...);
  if (nf == 1 && nb == 0) return F<1, 0>::go(a...);
  if (nf == 1 && nb == 2) return F<1, 2>::go(a...);
  if (nf == 2 && nb == 1) return F<2, 1>::go(a...);
  if (nf == 2 && nb == 0) return F<2, 0>::go(a...);
  if (nf == 2 && nb == 2) return F<2, 2>::go(a...);
  throw Error("unsupported group configuration: " + std::to_string(nf) + " fluid and " + std::to_string(nb) +
              " boundary groups (1..2 and 0..2 are supported)");
}

// A CUDA graph holding one conditional while node; the body is captured from
// the launches `body(stream, handle)` queues.  Rebuilt when the signature
// (the bytes of every kernel argument of the body) changes.
class WhileLoop {
public:
  ~WhileLoop() { reset(); }
  void reset() {
    if (exec_) cudaGraphExecDestroy(exec_);
    if (graph_) cudaGraphDestroy(graph_);
    exec_ = nullptr;
    graph_ = nullptr;
    sig_.clear();
  }
  template <class Body> void run(cudaStream_t s, std::string const &sig, Body &&body) {
    if (!exec_ || sig != sig_) {
      reset();
      PG_CUDA(cudaGraphCreate(&graph_, 0));
      cudaGraphConditionalHandle h;
      PG_CUDA(cudaGraphConditionalHandleCreate(&h, graph_, 1, cudaGraphCondAssignDefault));
      cudaGraphNodeParams p{};
      p.type = cudaGraphNodeTypeConditional;
      p.conditional.handle = h;
      p.conditional.type = cudaGraphCondTypeWhile;
      p.conditional.size = 1;
      cudaGraphNode_t node;
      PG_CUDA(cudaGraphAddNode(&node, graph_, nullptr, nullptr, 0, &p));
      cudaGraph_t bodyg = p.conditional.phGraph_out[0];
      cudaStream_t cs;
      PG_CUDA(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
      PG_CUDA(cudaStreamBeginCaptureToGraph(cs, bodyg, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
      uint64_t counted = launch_count();
      try {
        body(cs, h);
      } catch (...) {
        cudaGraph_t dummy;
        cudaStreamEndCapture(cs, &dummy);
        cudaStreamDestroy(cs);
        reset();
        throw;
      }
      uncount_launches(launch_count() - counted); // captured, not launched
      cudaGraph_t out;
      cudaError_t err = cudaStreamEndCapture(cs, &out);
      cudaStreamDestroy(cs);
      PG_CUDA(err);
      PG_CUDA(cudaGraphInstantiate(&exec_, graph_, 0));
      sig_ = sig;
      builds++;
    }
    PG_CUDA(cudaGraphLaunch(exec_, s));
  }
  int builds = 0;

private:
  cudaGraph_t graph_ = nullptr;
  cudaGraphExec_t exec_ = nullptr;
  std::string sig_;
};

template <class T> void sig_add(std::string &s, T const &v) { s.append(reinterpret_cast<char const *>(&v), sizeof(T)); }

} // namespace

// ===========================================================================
// Tuning knobs
// ===========================================================================

char const *tune_knob_name(int k) {
  static char const *names[kTuneKnobs] = {"density", "iisph_setup", "iisph_accel", "iisph_pressure",
                                          "wkbb18_diag", "pcg_init", "pcg_q", "jacobi_unroll", "staging",
                                          "grid_sort", "list_split"};
  return (k >= 0 && k < kTuneKnobs) ? names[k] : "";
}
int tune_knob_find(std::string const &name) {
  for (int k = 0; k < kTuneKnobs; ++k)
    if (name == tune_knob_name(k)) return k;
  return -1;
}
bool tune_value_ok(int k, int v) {
  if (k == kTuneJacobiUnroll) return v == 1 || v == 2 || v == 4;
  if (k == kTuneStaging || k == kTuneGridSort || k == kTuneListSplit) return v == 0 || v == 1;
  if (k == kTunePcgQ) return v >= 0 && v <= 4; // 4: the cell-tile sweep
  // 4: the persistent tiled sweeps of a batched model (work counter)
  if (k == kTuneAccel || k == kTunePressure) return v >= 0 && v <= 4;
  return k >= 0 && k < kTuneKnobs && v >= 0 && v <= 3;
}
std::string tune_knob_table() {
  // shapes as threads-per-block x blocks-per-SM / walk batch
  std::string t;
  t += "density 0 " + shapes_text<DensityShapes>() + "\n";
  t += "iisph_setup 0 " + shapes_text<SetupShapes>() + "\n";
  t += "iisph_accel 0 " + shapes_text<AccelShapes>() + " batched: " + shapes_text<AccelSegShapes>() +
       " 4=persistent tiles (batched; 0 otherwise)\n";
  t += "iisph_pressure 0 " + shapes_text<PressureShapes>() + " 4=persistent tiles (batched; 0 otherwise)\n";
  t += "wkbb18_diag 0 " + shapes_text<DiagShapes>() + "\n";
  t += "pcg_init 0 " + shapes_text<PcgShapes>() + "\n";
  t += "pcg_q 0 " + shapes_text<PcgShapes>() + " 4=cell-tiles (no lists; plain models)\n";
  t += "jacobi_unroll 1 1=1 2=2 4=4\n";
  t += "staging 0 0=off 1=staged lists and sweeps (unbatched models)\n";
  t += "grid_sort 1 0=tiled launches 1=one cluster launch for grids of at most 128k items\n";
  t += "list_split 1 0=one thread per query 1=four threads per query for query groups of at most 64k items\n";
  return t;
}

// ===========================================================================
// Scheme base
// ===========================================================================

void Scheme::run(std::string const &procedure, Nhood &nh, cudaStream_t s) {
  auto it = procs_.find(procedure);
  if (it == procs_.end()) throw Error("procedure does not exist");
  if (!model_) throw Error("scheme has not been loaded");
  it->second(nh, s);
}

std::vector<std::string> Scheme::procedure_names() const {
  std::vector<std::string> r;
  for (auto &kv : procs_) r.push_back(kv.first);
  return r;
}

uint64_t device_loop_kernels() {
  unsigned long long v = 0;
  if (cudaMemcpyFromSymbol(&v, g_loop_kernels, sizeof(v)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return uint64_t(v);
}

namespace {

// groups of a model selected by type / tag, with their fields
struct FluidG {
  Group *g;
  VaryingField *x, *v, *a, *rho, *p, *m, *c, *s, *AA, *Ap, *tb, *vd, *sp, *L;
  SmallField *rho0, *mu, *tol, *max_k, *iters;
};
struct BoundG {
  Group *g;
  VaryingField *x, *V;
  SmallField *mu;
};

class SchemeCommon : public Scheme {
protected:
  Globals globals(Model &m) {
    Globals G{};
    auto gp = [&](char const *n) -> void * {
      SmallField *f = m.find_global(n);
      return f ? m.small_ptr(*f) : nullptr;
    };
    G.h = static_cast<float const *>(gp("smoothing_scale"));
    G.dt = static_cast<float const *>(gp("time_step"));
    G.t = static_cast<float const *>(gp("current_time"));
    G.fade = static_cast<float const *>(gp("fade_duration"));
    G.omega = static_cast<float const *>(gp("iisph_relaxation"));
    G.aprde = static_cast<float *>(gp("iisph_aprde"));
    G.nprde = static_cast<int *>(gp("iisph_nprde"));
    G.gravity = static_cast<float const *>(gp("gravity"));
    G.max_speed = static_cast<float *>(gp("maximum_speed"));
    G.jac_max = static_cast<int const *>(gp("iisph_maximum_iterations"));
    G.jac_eta = static_cast<float const *>(gp("iisph_maximum_density_error"));
    G.jac_iters = static_cast<int *>(gp("iisph_iterations"));
    return G;
  }
  Red red(Model &m, int slot) {
    Red R;
    R.partials = m.red_d;
    R.ticket = m.red_count_d + slot;
    R.scalars = m.scalars_d;
    R.status = m.status_d;
    R.stats = m.stats_d;
    return R;
  }
  std::vector<FluidG> fluid_;
  std::vector<BoundG> bound_;

  // the per-slot view of a segmented group (batched models), or nullptr
  bool segmented(Group const *g) const { return model_->seg && model_->seg->find(g); }
  SegArgs seg_args(Group const *g) {
    Segments &S = *model_->seg;
    SegGroup const *G = S.find(g);
    if (!G) throw Error("group '" + g->name + "' has no segments");
    SegArgs a{};
    a.tiles = G->tiles;
    a.slot_tiles = G->slot_tiles;
    a.seg = G->seg;
    a.ntiles = G->ntiles;
    a.slots = S.slots;
    a.partials = S.partials;
    a.pcap = S.partial_cap;
    a.tickets = S.tickets;
    a.scal = S.scal;
    a.stat = S.stat;
    a.stats = S.stats;
    a.nprde = S.nprde;
    a.iters = S.iters;
    a.active = G->active;
    a.nactive = G->nactive;
    return a;
  }

  static NbrList nl(NbrView const &v, int g) { return NbrList{v.chunks[g], v.idx32[g], v.cb[g], v.cap[g], v.n}; }
  // packed neighbour records of the fluid / boundary groups (made current
  // here: may launch a pack kernel on `s`)
  FluidN fn(FluidG const &F, NbrView const &v, cudaStream_t s) {
    FluidN r{};
    r.L = nl(v, F.g->index);
    r.xm = model_->packed_xs(F.g, F.x, F.m, "xm", s);
    r.v = F.v ? dptr<float4>(F.v) : nullptr;
    r.a = F.a ? dptr<float4>(F.a) : nullptr;
    r.pr = nullptr;
    return r;
  }
  BoundN bn(BoundG const &B, NbrView const &v, cudaStream_t s) {
    BoundN r{};
    r.L = nl(v, B.g->index);
    r.xV = model_->packed_xs(B.g, B.x, B.V, "xV", s);
    r.mu = B.mu ? static_cast<float const *>(model_->small_ptr(*B.mu)) : nullptr;
    return r;
  }
  template <int NF, int NB> Nbrs<NF, NB> nbrs(NbrView const &v, cudaStream_t s) {
    Nbrs<NF, NB> N{};
    for (int q = 0; q < NF; ++q) N.f[q] = fn(fluid_[q], v, s);
    for (int q = 0; q < NB; ++q) N.b[q] = bn(bound_[q], v, s);
    N.hcache = v.hcache;
    return N;
  }
  template <int NB> Nbrs<0, NB> bnbrs(NbrView const &v, cudaStream_t s) {
    Nbrs<0, NB> N{};
    for (int q = 0; q < NB; ++q) N.b[q] = bn(bound_[q], v, s);
    N.hcache = v.hcache;
    return N;
  }
  // staged lists when the model's staging knob is on (fluid groups of an
  // unbatched model; the neighbourhood builds them only for the layouts the
  // staged sweeps handle)
  NbrView const &lists(Nhood &nh, Group *g, Globals const &G, cudaStream_t s) {
    bool stage = model_->tune.v[kTuneStaging] != 0 && g->type == "fluid" && !segmented(g);
    return nh.lists(g->index, s, G.h, stage);
  }
  // the staged sweeps' arguments for fluid group F (one fluid and one
  // boundary group, unbatched); false where the lists are not staged
  bool stage_args(Nhood &nh, NbrView const &v, FluidG const &F, StageArgs &SA) {
    if (!model_->tune.v[kTuneStaging] || fluid_.size() != 1 || bound_.size() != 1 || segmented(F.g)) return false;
    int fg = F.g->index, bg = bound_[0].g->index;
    if (!v.tile_info || !v.tile_cells || !v.slots[fg] || !v.slots[bg]) return false;
    SA = StageArgs{v.slots[fg], v.slots[bg], v.tile_info, v.tile_cells, nh.view().sorted, fg, bg};
    // per device and cheap: set on every solve (never inside a capture)
    static_assert(kStageSmem <= 64 * 1024, "staged records fit four blocks per SM");
    PG_CUDA(cudaFuncSetAttribute(k_iisph_accel_staged<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStageSmem)));
    PG_CUDA(cudaFuncSetAttribute(k_iisph_pressure_staged<16>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 int(kStageSmem)));
    PG_CUDA(cudaFuncSetAttribute(k_pcg_init_staged<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStageSmem)));
    PG_CUDA(cudaFuncSetAttribute(k_pcg_q_staged<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kStageSmem)));
    return true;
  }
  float const *u(SmallField *f) { return static_cast<float const *>(model_->small_ptr(*f)); }
  void need(std::initializer_list<std::pair<void const *, char const *>> l) {
    for (auto &p : l)
      if (!p.first) throw Error(std::string("global field missing: ") + p.second);
  }
  void collect(Model &m, bool fluid_fields, bool boundary_fields) {
    fluid_.clear();
    bound_.clear();
    for (Group *g : m.groups_by_index()) {
      if (g->type == "fluid" && fluid_fields) fluid_.push_back(FluidG{g});
      if (g->type == "boundary" && boundary_fields) bound_.push_back(BoundG{g});
    }
  }
};

// ---------------------------------------------------------------------------
// density
// ---------------------------------------------------------------------------

class Density : public SchemeCommon {
public:
  Density() { reg("compute_density", [this](Nhood &nh, cudaStream_t s) { compute_density(nh, s); }); }
  std::string name() const override { return "density"; }
  std::string source() const override {
    return "procedure compute_density: rho_f = sum_fluid m W(x_ff) + sum_boundary V rho0 W(x_fb)";
  }
  void load(Model &m) override {
    m.add_global("smoothing_scale", ft_real());
    collect(m, true, true);
    for (auto &F : fluid_) {
      F.rho0 = &F.g->add_uniform("rest_density", ft_real());
      F.x = &F.g->add_varying("position", ft_vec3());
      F.rho = &F.g->add_varying("density", ft_real());
      F.m = &F.g->add_varying("mass", ft_real());
    }
    for (auto &B : bound_) {
      B.x = &B.g->add_varying("position", ft_vec3());
      B.V = &B.g->add_varying("volume", ft_real());
    }
    bind(m);
  }
  template <int NF, int NB> struct L {
    static void go(Density *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, NB>(v, s);
      ProfScope ps(S->model_->prof, "density", s);
      with_shape<DensityShapes, NF == 1 && NB == 1>(S->model_->tune.v[kTuneDensity], [&](auto sh) {
        using Sh = decltype(sh);
        k_density<NF, NB, Sh::nt, Sh::minb, Sh::bt><<<div_up(n, Sh::nt), Sh::nt, 0, s>>>(
            n, dptr<float4>(F.x), dptr<float>(F.rho), S->u(F.rho0), G, N);
      });
      count_launch();
    }
  };
  void compute_density(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    for (auto &F : fluid_) {
      if (F.g->count == 0) continue;
      NbrView const &v = lists(nh, F.g, G, s);
      dispatch_fb<L>(int(fluid_.size()), int(bound_.size()), this, F, v, G, s);
      PG_LAUNCH_CHECK();
      F.rho->version++;
    }
  }
};

// ---------------------------------------------------------------------------
// aiast12
// ---------------------------------------------------------------------------

class Aiast12 : public SchemeCommon {
public:
  Aiast12() { reg("compute_volume", [this](Nhood &nh, cudaStream_t s) { compute_volume(nh, s); }); }
  std::string name() const override { return "aiast12"; }
  std::string source() const override { return "procedure compute_volume: V_b = 1 / sum_boundary W(x_bb)"; }
  void load(Model &m) override {
    m.add_global("smoothing_scale", ft_real());
    collect(m, false, true);
    for (auto &B : bound_) {
      B.x = &B.g->add_varying("position", ft_vec3());
      B.V = &B.g->add_varying("volume", ft_real());
    }
    bind(m);
  }
  void compute_volume(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    int nb = int(bound_.size());
    if (nb > 2) throw Error("unsupported group configuration: at most 2 boundary groups");
    // every group's sums read the positions before any volume is written
    std::vector<std::pair<BoundG *, NbrView const *>> todo;
    for (auto &B : bound_)
      if (B.g->count) todo.push_back({&B, &lists(nh, B.g, G, s)});
    for (auto &t : todo) {
      BoundG &B = *t.first;
      uint32_t n = uint32_t(B.g->count);
      NbrView const &v = *t.second;
      ProfScope ps(model_->prof, "aiast12_volume", s);
      if (nb == 1) {
        k_volume<1><<<div_up(n, kNT), kNT, 0, s>>>(n, dptr<float4>(B.x), dptr<float>(B.V), G, bnbrs<1>(v, s));
        count_launch();
      } else {
        k_volume<2><<<div_up(n, kNT), kNT, 0, s>>>(n, dptr<float4>(B.x), dptr<float>(B.V), G, bnbrs<2>(v, s));
        count_launch();
      }
      PG_LAUNCH_CHECK();
    }
    for (auto &t : todo) t.first->V->version++;
  }
};

// ---------------------------------------------------------------------------
// gravity / symplectic_euler (groups selected by the tag "dynamic")
// ---------------------------------------------------------------------------

class Gravity : public SchemeCommon {
public:
  Gravity() {
    reg("initialize_acceleration", [this](Nhood &, cudaStream_t s) {
      Globals G = globals(*model_);
      for (Group *g : dyn_) {
        uint32_t n = uint32_t(g->count);
        if (!n) continue;
        VaryingField *a = g->find_varying("acceleration");
        ProfScope ps(model_->prof, "gravity", s);
        k_gravity<<<div_up(n, 256), 256, 0, s>>>(n, dptr<float4>(a), G); count_launch();
        PG_LAUNCH_CHECK();
        a->version++;
      }
    });
  }
  std::string name() const override { return "gravity"; }
  std::string source() const override { return "procedure initialize_acceleration: a = g"; }
  void load(Model &m) override {
    m.add_global("gravity", ft_vec3());
    m.add_global("gravity_center", ft_vec3());
    dyn_.clear();
    for (Group *g : m.groups_by_index())
      if (g->has_tag("dynamic")) {
        g->add_varying("position", ft_vec3());
        g->add_varying("acceleration", ft_vec3());
        dyn_.push_back(g);
      }
    bind(m);
  }

private:
  std::vector<Group *> dyn_;
};

class SymplecticEuler : public SchemeCommon {
public:
  SymplecticEuler() {
    reg("integrate_velocity_with_hard_fade", [this](Nhood &, cudaStream_t s) {
      Globals G = globals(*model_);
      for (Group *g : dyn_) {
        uint32_t n = uint32_t(g->count);
        if (!n) continue;
        VaryingField *v = g->find_varying("velocity");
        ProfScope ps(model_->prof, "integrate_velocity", s);
        k_integrate_velocity<<<div_up(n, 256), 256, 0, s>>>(n, dptr<float4>(v),
                                                            dptr<float4>(g->find_varying("acceleration")),
                                                            dptr<float>(g->find_varying("time_of_birth")), G);
        count_launch();
        PG_LAUNCH_CHECK();
        v->version++;
      }
    });
    reg("integrate_position", [this](Nhood &, cudaStream_t s) {
      Globals G = globals(*model_);
      unsigned *maxord = reinterpret_cast<unsigned *>(model_->status_d + 8);
      k_max_speed_begin<<<1, 1, 0, s>>>(G, maxord); count_launch();
      for (Group *g : dyn_) {
        uint32_t n = uint32_t(g->count);
        if (!n) continue;
        VaryingField *x = g->find_varying("position");
        ProfScope ps(model_->prof, "integrate_position", s);
        k_integrate_position<<<div_up(n, 256), 256, 0, s>>>(n, dptr<float4>(x),
                                                            dptr<float4>(g->find_varying("velocity")), G, maxord);
        count_launch();
        x->version++;
      }
      k_max_speed_end<<<1, 1, 0, s>>>(G, maxord); count_launch();
      PG_LAUNCH_CHECK();
    });
  }
  std::string name() const override { return "symplectic_euler"; }
  std::string source() const override {
    return "procedures integrate_velocity_with_hard_fade: v += dt a [0 < t - t_birth - dt_fade]; "
           "integrate_position: x += dt v, max_speed max= |v|";
  }
  void load(Model &m) override {
    m.add_global("time_step", ft_real());
    m.add_global("current_time", ft_real());
    m.add_global("fade_duration", ft_real());
    m.add_global("maximum_speed", ft_real());
    dyn_.clear();
    for (Group *g : m.groups_by_index())
      if (g->has_tag("dynamic")) {
        g->add_varying("position", ft_vec3());
        g->add_varying("velocity", ft_vec3());
        g->add_varying("acceleration", ft_vec3());
        g->add_varying("time_of_birth", ft_real());
        dyn_.push_back(g);
      }
    bind(m);
  }

private:
  std::vector<Group *> dyn_;
};

// ---------------------------------------------------------------------------
// iisph
// ---------------------------------------------------------------------------

class Iisph : public SchemeCommon {
public:
  Iisph() {
    reg("setup", [this](Nhood &nh, cudaStream_t s) { setup(nh, s); });
    reg("iteration_pressure_acceleration", [this](Nhood &nh, cudaStream_t s) { accel(nh, s); });
    reg("iteration_pressure", [this](Nhood &nh, cudaStream_t s) { pressure(nh, s); });
    // the whole relaxed-Jacobi loop of the driver script on the device
    reg("solve_pressure", [this](Nhood &nh, cudaStream_t s) { solve(nh, s); });
  }
  std::string name() const override { return "iisph"; }
  std::string source() const override {
    return "procedures setup (c, p = 0, s, AA, nprde), iteration_pressure_acceleration (a), "
           "iteration_pressure (Ap, relaxed Jacobi p, aprde += (Ap - s) / rho0 [p > 1e-9]), "
           "solve_pressure (repeat aprde := 0, acceleration, pressure while the iteration count is < 2 or "
           "aprde / nprde >= iisph_maximum_density_error, at most iisph_maximum_iterations times)";
  }
  void load(Model &m) override {
    m.add_global("gravity", ft_vec3());
    m.add_global("smoothing_scale", ft_real());
    m.add_global("time_step", ft_real());
    m.add_global("iisph_relaxation", ft_real());
    m.add_global("iisph_aprde", ft_real());
    m.add_global("iisph_nprde", ft_int());
    m.add_global("iisph_maximum_iterations", ft_int());
    m.add_global("iisph_maximum_density_error", ft_real());
    m.add_global("iisph_iterations", ft_int());
    collect(m, true, true);
    for (auto &F : fluid_) {
      F.rho0 = &F.g->add_uniform("rest_density", ft_real());
      F.x = &F.g->add_varying("position", ft_vec3());
      F.v = &F.g->add_varying("velocity", ft_vec3());
      F.a = &F.g->add_varying("acceleration", ft_vec3());
      F.rho = &F.g->add_varying("density", ft_real());
      F.p = &F.g->add_varying("pressure", ft_real());
      F.m = &F.g->add_varying("mass", ft_real());
      F.c = &F.g->add_varying("iisph_helper_c", ft_vec3());
      F.s = &F.g->add_varying("iisph_source_term", ft_real());
      F.AA = &F.g->add_varying("iisph_diagonal_element", ft_real());
      F.Ap = &F.g->add_varying("iisph_right_hand_side", ft_real());
    }
    for (auto &B : bound_) {
      B.x = &B.g->add_varying("position", ft_vec3());
      B.V = &B.g->add_varying("volume", ft_real());
    }
    bind(m);
    loop_.reset();
  }
  template <int NF, int NB> struct SETUP {
    static void go(Iisph *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, NB>(v, s);
      float *pr = S->model_->pr_buffer(F.g, s);
      ProfScope ps(S->model_->prof, "iisph_setup", s);
      with_shape<SetupShapes, NF == 1 && NB == 1>(S->model_->tune.v[kTuneSetup], [&](auto sh) {
        using Sh = decltype(sh);
        k_iisph_setup<NF, NB, Sh::nt, Sh::minb, Sh::bt><<<div_up(n, Sh::nt), Sh::nt, 0, s>>>(
            n, dptr<float4>(F.x), dptr<float4>(F.v), dptr<float4>(F.c), dptr<float>(F.m), dptr<float>(F.rho),
            dptr<float>(F.p), pr, dptr<float>(F.s), dptr<float>(F.AA), S->u(F.rho0), G, N);
      });
      count_launch();
    }
  };
  // Pressure-acceleration / pressure launches of one group.  With `sig`
  // non-null nothing is launched: the kernel arguments are appended to the
  // signature of the device loop instead.  `done` is the loop flag
  // (nullptr outside the device loop); `prof` brackets the launch with
  // timing events (never on a capture stream).
  template <int NF, int NB> struct A {
    static void go(Iisph *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s, int const *done, bool prof,
                   std::string *sig, SegArgs const *SA = nullptr, StageArgs const *ST = nullptr) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, NB>(v, s);
      for (int q = 0; q < NF; ++q) N.f[q].pr = S->model_->packed_pr(S->fluid_[q].g, S->fluid_[q].p, S->fluid_[q].rho, s);
      float4 const *x = dptr<float4>(F.x);
      float const *p = dptr<float>(F.p), *rho = dptr<float>(F.rho);
      float4 *a = dptr<float4>(F.a);
      float const *rho0 = S->u(F.rho0);
      if (sig) {
        sig_add(*sig, n);
        sig_add(*sig, N);
        sig_add(*sig, x);
        sig_add(*sig, p);
        sig_add(*sig, rho);
        sig_add(*sig, a);
        sig_add(*sig, rho0);
        if (SA) sig_add(*sig, *SA);
        if (ST) sig_add(*sig, *ST);
        return;
      }
      if (prof) S->model_->prof.begin("iisph_accel", s);
      int tv = S->model_->tune.v[kTuneAccel];
      bool staged = false;
      if constexpr (NF == 1 && NB == 1) {
        if (ST && !SA) {
          k_iisph_accel_staged<8><<<div_up(n, kNT), kNT, kStageSmem, s>>>(n, x, p, rho, a, rho0, G, N, done, *ST);
          staged = true;
        }
      }
      if (staged) {
      } else if (SA) {
        if (SA->ntiles) {
          if (NF == 1 && NB == 1 && tv == 4)
            k_iisph_accel_seg<NF, NB, kMinBlocks, 8, true><<<std::min(SA->ntiles, kActiveBlocks), kNT, 0, s>>>(
                x, p, rho, a, rho0, G, N, *SA);
          else
            with_shape<AccelSegShapes, NF == 1 && NB == 1>(tv, [&](auto sh) {
              using Sh = decltype(sh);
              k_iisph_accel_seg<NF, NB, Sh::minb, Sh::bt><<<std::min(SA->ntiles, kActiveBlocks), kNT, 0, s>>>(
                  x, p, rho, a, rho0, G, N, *SA);
            });
        }
      } else {
        with_shape<AccelShapes, NF == 1 && NB == 1>(tv, [&](auto sh) {
          using Sh = decltype(sh);
          k_iisph_accel<NF, NB, Sh::nt, Sh::minb, Sh::bt><<<div_up(n, Sh::nt), Sh::nt, 0, s>>>(n, x, p, rho, a, rho0,
                                                                                            G, N, done);
        });
      }
      count_launch();
      if (prof) S->model_->prof.end(s);
    }
  };
  template <int NF, int NB> struct P {
    static void go(Iisph *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s, int first, int last,
                   int const *done, bool prof, std::string *sig, SegArgs const *SA = nullptr,
                   StageArgs const *ST = nullptr) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, NB>(v, s);
      float *pr = S->model_->pr_buffer(F.g, s);
      Red R = S->red(*S->model_, 0);
      PressureArgs PA{dptr<float4>(F.x), dptr<float4>(F.a), dptr<float>(F.rho), dptr<float>(F.s), dptr<float>(F.AA),
                      dptr<float>(F.p), pr, dptr<float>(F.Ap), S->u(F.rho0)};
      if (sig) {
        sig_add(*sig, n);
        sig_add(*sig, N);
        sig_add(*sig, R);
        sig_add(*sig, PA);
        sig_add(*sig, first);
        sig_add(*sig, last);
        if (SA) sig_add(*sig, *SA);
        if (ST) sig_add(*sig, *ST);
        return;
      }
      if (prof) S->model_->prof.begin("iisph_pressure", s);
      int tvp = S->model_->tune.v[kTunePressure];
      bool staged = false;
      if constexpr (NF == 1 && NB == 1) {
        if (ST && !SA) {
          k_iisph_pressure_staged<16><<<red_grid(n), kNT, kStageSmem, s>>>(n, PA, G, N, R, first, last, done, *ST);
          staged = true;
        }
      }
      if (staged) {
      } else if (SA && NF == 1 && NB == 1 && tvp == 4) {
        if (SA->ntiles)
          k_iisph_pressure_seg<NF, NB, kMinBlocks, 16, true><<<std::min(SA->ntiles, kActiveBlocks), kNT, 0, s>>>(
              PA, G, N, *SA);
      } else
      with_shape<PressureShapes, NF == 1 && NB == 1>(tvp, [&](auto sh) {
        using Sh = decltype(sh);
        if (SA) {
          if (SA->ntiles) k_iisph_pressure_seg<NF, NB, Sh::minb, Sh::bt><<<SA->ntiles, kNT, 0, s>>>(PA, G, N, *SA);
        } else {
          k_iisph_pressure<NF, NB, Sh::minb, Sh::bt><<<red_grid(n), kNT, 0, s>>>(n, PA, G, N, R, first, last, done);
        }
      });
      count_launch();
      if (prof) S->model_->prof.end(s);
    }
  };
  Globals checked_globals() {
    Globals G = globals(*model_);
    need({{G.h, "smoothing_scale"}, {G.dt, "time_step"}, {G.omega, "iisph_relaxation"}, {G.aprde, "iisph_aprde"},
          {G.nprde, "iisph_nprde"}, {G.jac_max, "iisph_maximum_iterations"}});
    return G;
  }
  std::vector<FluidG *> active() {
    std::vector<FluidG *> act;
    for (auto &F : fluid_)
      if (F.g->count) act.push_back(&F);
    return act;
  }
  // p and p / rho^2 were written together by a kernel
  void wrote_pressure(FluidG &F) {
    F.p->version++;
    model_->pack_commit(F.g, "pr", {uint64_t(F.g->count), reinterpret_cast<uint64_t>(F.p->d), F.p->version,
                                    reinterpret_cast<uint64_t>(F.rho->d), F.rho->version});
  }
  void setup(Nhood &nh, cudaStream_t s) {
    Globals G = checked_globals();
    int nf = int(fluid_.size()), nb = int(bound_.size());
    // one fused sweep per group (pass 2 of a group reads only its own c)
    long long total = 0;
    for (auto *F : active()) {
      total += (long long)F->g->count;
      dispatch_fb<SETUP>(nf, nb, this, *F, lists(nh, F->g, G, s), G, s);
      PG_LAUNCH_CHECK();
      F->c->version++;
      F->s->version++;
      F->AA->version++;
      wrote_pressure(*F);
    }
    // nprde = number of fluid particles (the generated reduction adds 1 per particle)
    k_set_i32<<<1, 1, 0, s>>>(G.nprde, int(total)); count_launch();
    PG_LAUNCH_CHECK();
  }
  void no_segments(char const *what) {
    for (auto &F : fluid_)
      if (segmented(F.g))
        throw Error(std::string(what) + " sums the density error over the whole group; on a batched (segmented) "
                    "model use solve_pressure, which decides convergence per scene");
  }
  void accel(Nhood &nh, cudaStream_t s) {
    no_segments("iteration_pressure_acceleration");
    Globals G = checked_globals();
    int nf = int(fluid_.size()), nb = int(bound_.size());
    for (auto *F : active()) {
      dispatch_fb<A>(nf, nb, this, *F, lists(nh, F->g, G, s), G, s, static_cast<int const *>(nullptr), true,
                     static_cast<std::string *>(nullptr));
      PG_LAUNCH_CHECK();
      F->a->version++;
    }
  }
  void pressure(Nhood &nh, cudaStream_t s) {
    no_segments("iteration_pressure");
    Globals G = checked_globals();
    int nf = int(fluid_.size()), nb = int(bound_.size());
    auto act = active();
    for (size_t k = 0; k < act.size(); ++k) {
      dispatch_fb<P>(nf, nb, this, *act[k], lists(nh, act[k]->g, G, s), G, s, k == 0 ? 1 : 0,
                     k + 1 == act.size() ? 1 : 0, static_cast<int const *>(nullptr), true,
                     static_cast<std::string *>(nullptr));
      PG_LAUNCH_CHECK();
      act[k]->Ap->version++;
      wrote_pressure(*act[k]);
    }
  }
  // The relaxed-Jacobi loop on the device: a CUDA graph whose conditional
  // while node repeats [acceleration, pressure, control] until the control
  // kernel clears the condition.  With profiling enabled the same kernels
  // are driven from the host, one iteration at a time, so that each launch
  // can be timed.
  void solve(Nhood &nh, cudaStream_t s) {
    Globals G = checked_globals();
    need({{G.jac_eta, "iisph_maximum_density_error"}, {G.jac_iters, "iisph_iterations"}});
    int nf = int(fluid_.size()), nb = int(bound_.size());
    auto act = active();
    Red R = red(*model_, 0);
    int const *done = R.status + kStJacDone;
    // batched model: one segmented fluid group, convergence per slot
    bool seg = false;
    for (auto &F : fluid_)
      if (segmented(F.g)) seg = true;
    SegArgs SA{};
    if (seg) {
      if (fluid_.size() != 1) throw Error("a batched model has exactly one fluid group");
      SA = seg_args(fluid_[0].g);
    }
    SegArgs const *sa = seg ? &SA : nullptr;
    // lists and packed records are made current before the loop, so that
    // building the loop launches nothing else
    std::vector<NbrView const *> views;
    for (auto *F : act) {
      views.push_back(&lists(nh, F->g, G, s));
      model_->packed_xs(F->g, F->x, F->m, "xm", s);
      model_->packed_pr(F->g, F->p, F->rho, s);
    }
    for (auto &B : bound_)
      if (B.g->count) model_->packed_xs(B.g, B.x, B.V, "xV", s);
    // staged sweeps (the staging knob): one fluid group, staged lists
    StageArgs st{};
    bool staged = !seg && act.size() == 1 && stage_args(nh, *views[0], *act[0], st);
    StageArgs const *stp = staged ? &st : nullptr;
    if (seg) {
      k_seg_jacobi_begin<<<div_up(std::max<uint32_t>(SA.slots, 1), 256), 256, 0, s>>>(SA); count_launch();
      k_seg_active<<<1, 1024, 0, s>>>(SA); count_launch();
      k_set_i32<<<1, 1, 0, s>>>(R.status + kStJacDone, 0); count_launch();
    } else {
      k_jacobi_begin<<<1, 1, 0, s>>>(G, R); count_launch();
    }
    PG_LAUNCH_CHECK();
    int kernels = 2 * int(act.size()) + 1;
    // iterations per graph iteration (the jacobi_unroll knob): the kernels of
    // the repeats after the control has ended the loop return at once, and
    // the last control of the body decides whether the body runs again
    int unroll = model_->tune.v[kTuneJacobiUnroll];
    auto body = [&](cudaStream_t cs, cudaGraphConditionalHandle h, bool use_handle, bool prof, std::string *sig) {
      int reps = (sig || prof) ? 1 : unroll;
      for (int rep = 0; rep < reps; ++rep) {
        for (size_t k = 0; k < act.size(); ++k)
          dispatch_fb<A>(nf, nb, this, *act[k], *views[k], G, cs, done, prof, sig, sa, stp);
        for (size_t k = 0; k < act.size(); ++k)
          dispatch_fb<P>(nf, nb, this, *act[k], *views[k], G, cs, k == 0 ? 1 : 0, k + 1 == act.size() ? 1 : 0, done,
                         prof, sig, sa, stp);
        if (sig) return;
        if (seg) {
          k_seg_jacobi_control<<<1, 1024, 0, cs>>>(G, SA, h, use_handle ? 1 : 0, use_handle ? kernels : 0,
                                                   R.status + kStJacDone);
        } else {
          k_jacobi_control<<<1, 1, 0, cs>>>(G, R, h, use_handle ? 1 : 0, use_handle ? kernels : 0);
        }
        count_launch();
      }
    };
    if (model_->prof.enabled) {
      // host-driven: one iteration per round trip
      for (int it = 0; it < 100000; ++it) {
        body(s, cudaGraphConditionalHandle{}, false, true, nullptr);
        PG_LAUNCH_CHECK();
        int d = 0;
        PG_CUDA(cudaMemcpyAsync(&d, done, sizeof(int), cudaMemcpyDeviceToHost, s));
        PG_CUDA(cudaStreamSynchronize(s));
        if (d) break;
      }
    } else {
      std::string sig;
      body(s, cudaGraphConditionalHandle{}, true, false, &sig);
      sig_add(sig, G);
      sig_add(sig, R);
      sig_add(sig, model_->tune); // a changed shape or repeat count rebuilds the graph
      loop_.run(s, sig, [&](cudaStream_t cs, cudaGraphConditionalHandle h) { body(cs, h, true, false, nullptr); });
      PG_LAUNCH_CHECK();
    }
    for (auto *F : act) {
      F->a->version++;
      F->Ap->version++;
      wrote_pressure(*F);
    }
  }

private:
  WhileLoop loop_;
};

// ---------------------------------------------------------------------------
// wkbb18
// ---------------------------------------------------------------------------

// gc: wkbb18_gc (share/schemes/wkbb18_gc.prtcl), the same procedures with
// every kernel gradient premultiplied by the item's gradient correction
class Wkbb18 : public SchemeCommon {
public:
  explicit Wkbb18(bool gc = false) : gc_(gc) {
    reg("compute_diagonal", [this](Nhood &nh, cudaStream_t s) { diag(nh, s); });
    reg("accumulate_acceleration", [this](Nhood &nh, cudaStream_t s) { pcg(nh, s); });
  }
  ~Wkbb18() override { free_vectors(); }
  std::string name() const override { return gc_ ? "wkbb18_gc" : "wkbb18"; }
  std::string source() const override {
    return std::string("procedures compute_diagonal (sp = (I - dt S)^-1), accumulate_acceleration (PCG over fluid "
                       "velocities with the implicit viscosity system, Jacobi block preconditioner sp, apply vd and "
                       "a = vd / dt)") +
           (gc_ ? "; every kernel gradient premultiplied by gradient_correction" : "");
  }
  void load(Model &m) override {
    m.add_global("smoothing_scale", ft_real());
    m.add_global("time_step", ft_real());
    m.add_global("current_time", ft_real());
    m.add_global("fade_duration", ft_real());
    collect(m, true, true);
    for (auto &F : fluid_) {
      F.rho0 = &F.g->add_uniform("rest_density", ft_real());
      F.mu = &F.g->add_uniform("dynamic_viscosity", ft_real());
      F.tol = &F.g->add_uniform("wkbb18_maximum_error", ft_real());
      F.max_k = &F.g->add_uniform("wkbb18_maximum_iterations", ft_int());
      F.iters = &F.g->add_uniform("wkbb18_iterations", ft_int());
      F.x = &F.g->add_varying("position", ft_vec3());
      F.v = &F.g->add_varying("velocity", ft_vec3());
      F.a = &F.g->add_varying("acceleration", ft_vec3());
      F.rho = &F.g->add_varying("density", ft_real());
      F.m = &F.g->add_varying("mass", ft_real());
      F.vd = &F.g->add_varying("wkbb18_velocity_delta", ft_vec3());
      F.sp = &F.g->add_varying("wkbb18_system_diagonal", ft_mat3());
      F.tb = &F.g->add_varying("time_of_birth", ft_real());
      F.L = gc_ ? &F.g->add_varying("gradient_correction", ft_mat3()) : nullptr;
    }
    for (auto &B : bound_) {
      B.mu = &B.g->add_uniform("dynamic_viscosity", ft_real());
      B.x = &B.g->add_varying("position", ft_vec3());
      B.V = &B.g->add_varying("volume", ft_real());
    }
    bind(m);
    loops_.clear();
  }
  template <int NB> void diag_launch(FluidG &F, NbrView const &v, Globals G, cudaStream_t s) {
    uint32_t n = uint32_t(F.g->count);
    auto N = bnbrs<NB>(v, s);
    float4 const *xmr = model_->packed_xmr(F.g, F.x, F.m, F.rho, s);
    ProfScope ps(model_->prof, "wkbb18_diag", s);
    if (gc_)
      k_wkbb18_diag<NB, true><<<div_up(n, kNT), kNT, 0, s>>>(n, uint32_t(F.sp->cap), xmr, dptr<float>(F.rho),
                                                              dptr<float>(F.sp), u(F.rho0), u(F.mu), G,
                                                              nl(v, F.g->index), N, dptr<float>(F.L),
                                                              uint32_t(F.L->cap));
    else
      with_shape<DiagShapes, NB == 1>(fluid_.size() == 1 ? model_->tune.v[kTuneDiag] : 0, [&](auto sh) {
        using Sh = decltype(sh);
        k_wkbb18_diag<NB, false, Sh::nt, Sh::minb, Sh::bt><<<div_up(n, Sh::nt), Sh::nt, 0, s>>>(
            n, uint32_t(F.sp->cap), xmr, dptr<float>(F.rho), dptr<float>(F.sp), u(F.rho0), u(F.mu), G,
            nl(v, F.g->index), N, nullptr, 0u);
      });
    count_launch();
  }
  void diag(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    int nb = int(bound_.size());
    for (auto &F : fluid_) {
      if (!F.g->count) continue;
      NbrView const &v = lists(nh, F.g, G, s);
      if (nb == 0) diag_launch<0>(F, v, G, s);
      else if (nb == 1) diag_launch<1>(F, v, G, s);
      else if (nb == 2) diag_launch<2>(F, v, G, s);
      else throw Error("unsupported group configuration: at most 2 boundary groups");
      PG_LAUNCH_CHECK();
      F.sp->version++;
    }
  }

  // solver/cg_openmp.hpp:35-215 on the device: guess and initial residual,
  // then a device loop of [q = A p, update, p update, control], then apply
  template <int NB> void pcg_group(FluidG &F, NbrView const &v, Globals G, cudaStream_t s, Nhood &nh) {
    if (gc_) pcg_group_t<NB, true>(F, v, G, s, nh);
    else pcg_group_t<NB, false>(F, v, G, s, nh);
  }
  template <int NB, bool GC> void pcg_group_t(FluidG &F, NbrView const &v, Globals G, cudaStream_t s, Nhood &nh) {
    uint32_t n = uint32_t(F.g->count);
    ensure_vectors(n);
    PcgArgs P{};
    P.n = n;
    P.cap = uint32_t(F.sp->cap);
    P.xmr = model_->packed_xmr(F.g, F.x, F.m, F.rho, s);
    P.v = dptr<float4>(F.v);
    P.rho = dptr<float>(F.rho);
    P.sp = dptr<float>(F.sp);
    P.tb = dptr<float>(F.tb);
    P.vd = dptr<float4>(F.vd);
    P.a = dptr<float4>(F.a);
    P.X = vec_[0];
    P.Y = vec_[1];
    P.Rr = vec_[2];
    P.P = vec_[3];
    P.Q = vec_[4];
    P.rho0 = u(F.rho0);
    P.mu = u(F.mu);
    P.tol = u(F.tol);
    P.max_k = static_cast<int const *>(model_->small_ptr(*F.max_k));
    P.iterations = static_cast<int *>(model_->small_ptr(*F.iters));
    P.self = nl(v, F.g->index);
    P.L = GC ? dptr<float>(F.L) : nullptr;
    P.lcap = GC ? uint32_t(F.L->cap) : 0u;
    auto N = bnbrs<NB>(v, s);
    Red R = red(*model_, 1);
    unsigned rg = red_grid(n), eg = div_up(n, 256);
    // batched model: one PCG per slot
    bool seg = segmented(F.g);
    SegArgs SA = seg ? seg_args(F.g) : SegArgs{};
    unsigned tg = SA.ntiles;
    k_pcg_guess<<<eg, 256, 0, s>>>(P); count_launch();
    constexpr bool kTuned = NB == 1 && !GC;
    int tv_init = fluid_.size() == 1 ? model_->tune.v[kTunePcgInit] : 0;
    int tv_q = fluid_.size() == 1 ? model_->tune.v[kTunePcgQ] : 0;
    // staged sweeps (the staging knob) for the tuned layout, except with the
    // cell-tile sweep
    StageArgs st{};
    bool staged = false;
    if constexpr (kTuned) staged = !seg && tv_q != 4 && stage_args(nh, v, F, st);
    {
      ProfScope ps(model_->prof, "pcg_init", s);
      if (seg) {
        k_seg_pcg_begin<<<div_up(std::max<uint32_t>(SA.slots, 1), 256), 256, 0, s>>>(SA); count_launch();
      }
      if constexpr (kTuned)
        if (staged) k_pcg_init_staged<8><<<rg, kNT, kStageSmem, s>>>(P, G, N, R, st);
      if (!staged)
      with_shape<PcgShapes, kTuned>(tv_init, [&](auto sh) {
        using Sh = decltype(sh);
        if (seg) {
          if (tg) k_pcg_init_seg<NB, GC, Sh::minb, Sh::bt><<<tg, kNT, 0, s>>>(P, G, N, SA);
        } else {
          k_pcg_init<NB, GC, Sh::minb, Sh::bt><<<rg, kNT, 0, s>>>(P, G, N, R);
        }
      });
      count_launch();
    }
    PG_LAUNCH_CHECK();
    // shape 4 of pcg_q: the cell-tile sweep (plain models of the tuned layout)
    bool tiles = false;
    GridView gv{};
    float4 const *xs = nullptr;
    int fg = F.g->index, bg = bound_.empty() ? -1 : bound_[0].g->index;
    if constexpr (kTuned) {
      gv = nh.view();
      // the tiles walk the grid's cells: the fluid group must be in the grid
      if (!seg && tv_q == 4 && gv.in_grid[fg]) {
        tiles = true;
        xs = nh.sorted_positions();
        // per device and cheap: set on every solve (never inside a capture)
        PG_CUDA(cudaFuncSetAttribute(k_pcg_q_tiles<NB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     int(2 * kTileStage * sizeof(float4))));
      }
    }
    auto body = [&](cudaStream_t cs, cudaGraphConditionalHandle h, bool use_handle, bool prof) {
      if (prof) model_->prof.begin("pcg_q", cs);
      if constexpr (kTuned) {
        if (tiles)
          k_pcg_q_tiles<NB><<<rg, kNT, 2 * kTileStage * sizeof(float4), cs>>>(P, G, N, R, gv, xs, fg, bg);
        else if (staged)
          k_pcg_q_staged<8><<<rg, kNT, kStageSmem, cs>>>(P, G, N, R, st);
      }
      if (!tiles && !staged)
        with_shape<PcgShapes, kTuned>(tv_q, [&](auto sh) {
          using Sh = decltype(sh);
          if (seg) {
            if (tg) k_pcg_q_seg<NB, GC, Sh::minb, Sh::bt><<<tg, kNT, 0, cs>>>(P, G, N, SA);
          } else {
            k_pcg_q<NB, GC, Sh::minb, Sh::bt><<<rg, kNT, 0, cs>>>(P, G, N, R);
          }
        });
      count_launch();
      if (prof) model_->prof.end(cs);
      if (prof) model_->prof.begin("pcg_update", cs);
      if (seg) {
        if (tg) k_pcg_update_seg<<<tg, kSegUpdateNT, 0, cs>>>(P, SA);
      } else {
        // one resident wave: each thread folds several items before the
        // block's FP64 tree (the FP64 pipe is narrow on this GPU)
        k_pcg_update<<<std::min(rg, unsigned(152 * kMinBlocks)), kNT, 0, cs>>>(P, R);
      }
      count_launch();
      if (prof) model_->prof.end(cs);
      if (prof) model_->prof.begin("pcg_p", cs);
      if (seg) k_pcg_p_seg<<<eg, 256, 0, cs>>>(P, SA);
      else k_pcg_p<<<rg, kNT, 0, cs>>>(P, R);
      count_launch();
      if (prof) model_->prof.end(cs);
      if (seg)
        k_seg_pcg_control<<<1, 1024, 0, cs>>>(P, SA, h, use_handle ? 1 : 0, use_handle ? 4 : 0,
                                              R.status + kStPcgActive);
      else
        k_pcg_control<<<1, 1, 0, cs>>>(P, R, h, use_handle ? 1 : 0, use_handle ? 4 : 0);
      count_launch();
    };
    if (model_->prof.enabled) {
      // host-driven (timed launches): one iteration per round trip
      for (int it = 0; it < 1000000; ++it) {
        body(s, cudaGraphConditionalHandle{}, false, true);
        PG_LAUNCH_CHECK();
        int active = 0;
        PG_CUDA(cudaMemcpyAsync(&active, R.status + kStPcgActive, sizeof(int), cudaMemcpyDeviceToHost, s));
        PG_CUDA(cudaStreamSynchronize(s));
        if (!active) break;
      }
    } else {
      std::string sig;
      sig_add(sig, P);
      sig_add(sig, N);
      sig_add(sig, R);
      sig_add(sig, G);
      sig_add(sig, rg);
      sig_add(sig, SA);
      sig_add(sig, model_->tune); // a changed shape rebuilds the graph
      if (tiles) {
        sig_add(sig, gv);
        sig_add(sig, xs);
      }
      if (staged) sig_add(sig, st);
      loops_[F.g].run(s, sig, [&](cudaStream_t cs, cudaGraphConditionalHandle h) { body(cs, h, true, false); });
      PG_LAUNCH_CHECK();
    }
    Red RA = R;
    if (seg) RA.status = nullptr; // per-slot iteration counts are in the segments' state
    k_pcg_apply<<<eg, 256, 0, s>>>(P, G, RA); count_launch();
    PG_LAUNCH_CHECK();
    F.vd->version++;
    F.a->version++;
  }
  void pcg(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    int nb = int(bound_.size());
    for (auto &F : fluid_) {
      if (!F.g->count) {
        int zero = 0;
        model_->small_set(*F.iters, &zero, s);
        continue;
      }
      NbrView const &v = lists(nh, F.g, G, s);
      if (nb == 0) pcg_group<0>(F, v, G, s, nh);
      else if (nb == 1) pcg_group<1>(F, v, G, s, nh);
      else if (nb == 2) pcg_group<2>(F, v, G, s, nh);
      else throw Error("unsupported group configuration: at most 2 boundary groups");
    }
  }

private:
  bool gc_;
  float4 *vec_[5] = {};
  size_t vec_cap_ = 0;
  std::map<Group *, WhileLoop> loops_;
  void free_vectors() {
    for (auto &p : vec_)
      if (p) {
        cudaFree(p);
        p = nullptr;
      }
    vec_cap_ = 0;
  }
  void ensure_vectors(size_t n) {
    if (n <= vec_cap_) return;
    loops_.clear(); // the captured loops hold the old vectors
    free_vectors();
    for (auto &p : vec_) PG_CUDA(cudaMalloc(&p, n * 16));
    vec_cap_ = n;
  }
};

// ---------------------------------------------------------------------------
// viscosity (explicit)
// ---------------------------------------------------------------------------

class Viscosity : public SchemeCommon {
public:
  Viscosity() {
    reg("accumulate_acceleration", [this](Nhood &nh, cudaStream_t s) { accumulate(nh, s); });
  }
  std::string name() const override { return "viscosity"; }
  std::string source() const override {
    return "procedure accumulate_acceleration: a_f += 10 (mu_f / rho_f) (m_f' / rho_f') (v_f - v_f').x_ff' / "
           "(|x_ff'|^2 + 0.01 h^2) gradW + boundary term with v_b = 0";
  }
  void load(Model &m) override {
    m.add_global("smoothing_scale", ft_real());
    collect(m, true, true);
    for (auto &F : fluid_) {
      F.rho0 = &F.g->add_uniform("rest_density", ft_real());
      F.mu = &F.g->add_uniform("dynamic_viscosity", ft_real());
      F.x = &F.g->add_varying("position", ft_vec3());
      F.v = &F.g->add_varying("velocity", ft_vec3());
      F.a = &F.g->add_varying("acceleration", ft_vec3());
      F.rho = &F.g->add_varying("density", ft_real());
      F.m = &F.g->add_varying("mass", ft_real());
    }
    for (auto &B : bound_) {
      B.mu = &B.g->add_uniform("dynamic_viscosity", ft_real());
      B.x = &B.g->add_varying("position", ft_vec3());
      B.V = &B.g->add_varying("volume", ft_real());
    }
    bind(m);
  }
  template <int NF, int NB> struct L {
    static void go(Viscosity *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, NB>(v, s);
      // fluid neighbour records (x, m / rho)
      for (int q = 0; q < NF; ++q) {
        FluidG &Q = S->fluid_[q];
        N.f[q].xm = S->model_->packed_xmr(Q.g, Q.x, Q.m, Q.rho, s);
      }
      ProfScope ps(S->model_->prof, "viscosity", s);
      k_viscosity<NF, NB><<<div_up(n, kNT), kNT, 0, s>>>(n, dptr<float4>(F.x), dptr<float4>(F.v), dptr<float>(F.rho),
                                                          dptr<float4>(F.a), S->u(F.rho0), S->u(F.mu), G, N);
      count_launch();
    }
  };
  void accumulate(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    need({{G.h, "smoothing_scale"}});
    // every group's sums read the accelerations of no neighbour: groups in turn
    for (auto &F : fluid_) {
      if (!F.g->count) continue;
      NbrView const &v = lists(nh, F.g, G, s);
      dispatch_fb<L>(int(fluid_.size()), int(bound_.size()), this, F, v, G, s);
      PG_LAUNCH_CHECK();
      F.a->version++;
    }
  }
};

// ---------------------------------------------------------------------------
// correction (gradient correction for wkbb18_gc)
// ---------------------------------------------------------------------------

class Correction : public SchemeCommon {
public:
  Correction() {
    reg("identity_gradient_correction", [this](Nhood &, cudaStream_t s) {
      for (auto &F : fluid_) {
        uint32_t n = uint32_t(F.g->count);
        if (!n) continue;
        k_identity9<<<div_up(n, 256), 256, 0, s>>>(n, uint32_t(F.L->cap), dptr<float>(F.L));
        count_launch();
        PG_LAUNCH_CHECK();
        F.L->version++;
      }
    });
    reg("compute_gradient_correction", [this](Nhood &nh, cudaStream_t s) { compute(nh, s); });
  }
  std::string name() const override { return "correction"; }
  std::string source() const override {
    return "procedures identity_gradient_correction (L = I), compute_gradient_correction (L_f = invert_pm(sum_fluid "
           "(m_f' / rho_f) gradW(x_ff') (x_f' - x_f)^T))";
  }
  void load(Model &m) override {
    m.add_global("smoothing_scale", ft_real());
    collect(m, true, false);
    for (auto &F : fluid_) {
      F.x = &F.g->add_varying("position", ft_vec3());
      F.rho = &F.g->add_varying("density", ft_real());
      F.m = &F.g->add_varying("mass", ft_real());
      F.L = &F.g->add_varying("gradient_correction", ft_mat3());
    }
    bind(m);
  }
  template <int NF, int NB> struct L {
    static void go(Correction *S, FluidG &F, NbrView const &v, Globals G, cudaStream_t s) {
      uint32_t n = uint32_t(F.g->count);
      auto N = S->nbrs<NF, 0>(v, s);
      ProfScope ps(S->model_->prof, "correction", s);
      k_correction<NF, 0><<<div_up(n, kNT), kNT, 0, s>>>(n, uint32_t(F.L->cap), dptr<float4>(F.x), dptr<float>(F.rho),
                                                          dptr<float>(F.L), G, N);
      count_launch();
    }
  };
  void compute(Nhood &nh, cudaStream_t s) {
    Globals G = globals(*model_);
    need({{G.h, "smoothing_scale"}});
    // every group's sums read positions, masses and densities only
    for (auto &F : fluid_) {
      if (!F.g->count) continue;
      NbrView const &v = lists(nh, F.g, G, s);
      dispatch_fb<L>(int(fluid_.size()), 0, this, F, v, G, s);
      PG_LAUNCH_CHECK();
      F.L->version++;
    }
  }
};

using Factory = std::unique_ptr<Scheme> (*)();

std::unique_ptr<Scheme> make_wkbb18_gc() { return std::unique_ptr<Scheme>(new Wkbb18(true)); }

template <class S> std::unique_ptr<Scheme> make() { return std::unique_ptr<Scheme>(new S()); }

std::map<std::string, Factory> const &registry() {
  static std::map<std::string, Factory> r = [] {
    std::map<std::string, Factory> m;
    auto add = [&](Factory f) { m[f()->full_name()] = f; };
    add(&make<Aiast12>);
    add(&make<Density>);
    add(&make<Gravity>);
    add(&make<Iisph>);
    add(&make<SymplecticEuler>);
    add(&make<Wkbb18>);
    add(&make<Viscosity>);
    add(&make<Correction>);
    add(&make_wkbb18_gc);
    return m;
  }();
  return r;
}

} // namespace

namespace {
std::map<std::string, SchemeFactory> &added() {
  static std::map<std::string, SchemeFactory> m;
  return m;
}
} // namespace

void register_scheme(std::string const &full_name, SchemeFactory f) {
  if (registry().count(full_name) || added().count(full_name))
    throw Error("scheme is already registered: " + full_name);
  added()[full_name] = std::move(f);
}

std::unique_ptr<Scheme> new_scheme(std::string const &full_name) {
  auto const &r = registry();
  auto it = r.find(full_name);
  if (it != r.end()) return it->second();
  auto jt = added().find(full_name);
  if (jt != added().end()) return jt->second();
  throw Error("scheme is not registered");
}

std::vector<std::string> scheme_names() {
  std::vector<std::string> v;
  for (auto &kv : registry()) v.push_back(kv.first);
  for (auto &kv : added()) v.push_back(kv.first);
  return v;
}

} // namespace prtcl_gpu
