// Shared helpers of the GB300 SPH hot path: error handling, the exact-order
// FP32 vector arithmetic and the cubic spline kernel used by every procedure.
//
// Every translation unit of this library is compiled with -fmad=false and
// IEEE division / square root, so that each expression below rounds exactly
// like the reference's scalar x86-64 code (no fused multiply-add) and the
// per-particle results reproduce the CPU restatement bit for bit.
#pragma once

#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <limits>
#include <stdexcept>
#include <string>

namespace prtcl_gpu {

struct Error : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define PG_CUDA(call)                                                                  \
  do {                                                                                 \
    cudaError_t e_ = (call);                                                           \
    if (e_ != cudaSuccess)                                                             \
      throw ::prtcl_gpu::Error(std::string("CUDA error: ") + cudaGetErrorString(e_) +  \
                               " at " + __FILE__ + ":" + std::to_string(__LINE__));    \
  } while (0)

#define PG_LAUNCH_CHECK() PG_CUDA(cudaGetLastError())

constexpr int kMaxGroups = 16;    // 4 group bits in a grid handle
constexpr int kMaxNbrGroups = 4;  // fluid / boundary groups a procedure sums over

inline unsigned div_up(size_t a, size_t b) { return unsigned((a + b - 1) / b); }

// float -> double from the two IEEE-754 binary formats, on the integer pipe:
// the conversion is exact, so the value equals the hardware conversion's
// (a NaN keeps its payload bits).  The FP64 reductions convert one float per
// item; GB300's FP64 pipe is narrow, so it is kept for the additions.
__host__ __device__ __forceinline__ double f2d(float f) {
#ifdef __CUDA_ARCH__
  uint32_t u = __float_as_uint(f);
#else
  uint32_t u;
  __builtin_memcpy(&u, &f, 4);
#endif
  uint64_t bits = uint64_t(u & 0x80000000u) << 32;
  uint32_t e = (u >> 23) & 0xFFu, m = u & 0x7FFFFFu;
  if (e == 0xFFu) {
    bits |= 0x7FF0000000000000ull | (uint64_t(m) << 29);
  } else if (e != 0u) {
    bits |= (uint64_t(e + (1023u - 127u)) << 52) | (uint64_t(m) << 29);
  } else if (m != 0u) {
    // subnormal m * 2^-149, leading one at bit p: a normal double
#ifdef __CUDA_ARCH__
    int p = 31 - __clz(int(m));
#else
    int p = 31 - __builtin_clz(m);
#endif
    bits |= (uint64_t(p + (1023 - 149)) << 52) | ((uint64_t(m) << (52 - p)) & 0x000FFFFFFFFFFFFFull);
  }
#ifdef __CUDA_ARCH__
  return __longlong_as_double((long long)bits);
#else
  double d;
  __builtin_memcpy(&d, &bits, 8);
  return d;
#endif
}

// number of kernels this library has launched from the host (process-wide)
uint64_t launch_count();
void count_launch();
void uncount_launches(uint64_t n);
// kernels executed inside device-side loops (CUDA graph bodies); reads a
// device counter
uint64_t device_loop_kernels();

// ---------------------------------------------------------------------------
// FP32 vector helpers in the reference's evaluation order
// ---------------------------------------------------------------------------

struct f3 {
  float x, y, z;
};

__device__ __forceinline__ f3 mk3(float4 v) { return {v.x, v.y, v.z}; }
__device__ __forceinline__ f3 sub3(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 add3(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 scl3(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
// a0*b0 + (a1*b1 + a2*b2): the unrolled 3-term reduction of the reference's
// tensor library
__device__ __forceinline__ float dot3(f3 a, f3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ float nsq3(f3 a) { return dot3(a, a); }

// unit_step_l (math/impl/eigen.hpp:307-314) and reciprocal_or_zero (:293-300)
__device__ __forceinline__ float ustep(float eps, float x) { return (eps < x) ? 1.0f : 0.0f; }
__device__ __forceinline__ float rcp0(float x, float eps) { return (fabsf(x) > eps) ? 1.0f / x : 0.0f; }

// ---------------------------------------------------------------------------
// cubic spline kernel with support 2h
// (math/kernel/cubic_spline_kernel.hpp:43-102, kernel_facade.hpp:95-120)
// ---------------------------------------------------------------------------

struct KernelParams {
  float h;      // smoothing scale
  float h3;     // ((h*h)*h), the reference's constpow(h, 3)
  float h4;     // (((h*h)*h)*h)
  float sigma;  // 1/(4 pi) rounded to f32
  float eps;    // sqrt(FLT_EPSILON): gradient is zero below this distance
};

inline KernelParams make_kernel_params(float h) {
  KernelParams k;
  k.h = h;
  volatile float a = h * h; // keep the host compiler from re-associating
  volatile float b = a * h;
  k.h3 = b;
  volatile float c = b * h;
  k.h4 = c;
  k.sigma = static_cast<float>(0.25L * 0.318309886183790671537767526745028724L);
  k.eps = std::sqrt(std::numeric_limits<float>::epsilon()); // math/constants.hpp:76-77
  return k;
}

// the kernel parameters for smoothing scale h, computed on the device with
// the same operations as the reference's constpow
__device__ __forceinline__ KernelParams kparams(float h) {
  KernelParams k;
  k.h = h;
  k.h3 = (h * h) * h;
  k.h4 = ((h * h) * h) * h;
  k.sigma = 0.0795774715459476678844418816862571810f; // 1/(4 pi) rounded to f32
  k.eps = 3.4526698300124390840e-04f;                 // sqrt(FLT_EPSILON)
  return k;
}

__device__ __forceinline__ float k_evalq(KernelParams const &k, float q) {
  float result = 0.0f;
  if (q < 1.0f) {
    float t = 1.0f - q;
    result -= 4.0f * ((t * t) * t);
  }
  if (q < 2.0f) {
    float t = 2.0f - q;
    result += (t * t) * t;
  }
  return k.sigma * result;
}
__device__ __forceinline__ float k_evaldq(KernelParams const &k, float q) {
  float result = 0.0f;
  if (q < 1.0f) {
    float t = 1.0f - q;
    result += 12.0f * (t * t);
  }
  if (q < 2.0f) {
    float t = 2.0f - q;
    result -= 3.0f * (t * t);
  }
  return k.sigma * result;
}
__device__ __forceinline__ float kW(KernelParams const &k, f3 v) {
  float r = sqrtf(nsq3(v));
  return k_evalq(k, fabsf(r) / k.h) / k.h3;
}
__device__ __forceinline__ f3 kgradW(KernelParams const &k, f3 v) {
  float r = sqrtf(nsq3(v));
  if (r < k.eps) return {0.0f, 0.0f, 0.0f};
  float dr = -copysignf(k_evaldq(k, fabsf(r) / k.h) / k.h4, r);
  return scl3(dr / r, v);
}

// The scalar factor of kgradW for a pair with squared distance d2:
// gradW(v) = factor * v.  +0.0 encodes the exactly-zero gradient below eps;
// any other factor is <= -0.0, so the encoding is unique.
__device__ __forceinline__ float kgrad_factor(KernelParams const &k, float d2) {
  float r = sqrtf(d2);
  if (r < k.eps) return 0.0f;
  float dr = -copysignf(k_evaldq(k, fabsf(r) / k.h) / k.h4, r);
  return dr / r;
}
// gradW from a cached factor, bit-identical to kgradW(k, v)
__device__ __forceinline__ f3 kgrad_from(float factor, f3 v) {
  if (__float_as_uint(factor) == 0u) return {0.0f, 0.0f, 0.0f};
  return scl3(factor, v);
}

// ---------------------------------------------------------------------------
// block reductions
// ---------------------------------------------------------------------------

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  return v;
}

// sum over a block of blockDim.x (multiple of 32, <= 1024) threads in a fixed
// tree order; the result is valid in thread 0
__device__ __forceinline__ double block_sum(double v, double *sh /* >= 32 */) {
  v = warp_sum(v);
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  if (lane == 0) sh[w] = v;
  __syncthreads();
  double r = 0.0;
  if (w == 0) {
    int nw = blockDim.x >> 5;
    r = (lane < nw) ? sh[lane] : 0.0;
    r = warp_sum(r);
  }
  __syncthreads();
  return r;
}

} // namespace prtcl_gpu
