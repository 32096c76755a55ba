// Device side of the schemes generated from the scheme language
// (prtcl_gb300/dsl): value types, the operators and functions of the
// language with the operation order of the reference's generated C++
// (prtcl::math over Eigen, math/impl/eigen.hpp:124-345, math/common.hpp,
// math/kernel.hpp, math/kernel/kernel_facade.hpp:95-120, math/aat13.hpp),
// and accessors of the model's field storage.
//
// Types: real -> float, real[] -> f3, real[][] -> M3 (column-major),
// integer -> int.  Sums of three terms (dot, norms, matrix products, trace)
// associate as a0 + (a1 + a2), the order the hand-written kernels and the
// oracle use for Eigen's fixed-size reductions.
#pragma once

#include "mat3.cuh"
#include "nbr_walk.cuh"

#include <cmath>

namespace prtcl_gpu {
namespace dsl {

using prtcl_gpu::f3;
using prtcl_gpu::M3;

// ---- vector operators (componentwise, like Eigen's expressions)
__device__ __forceinline__ f3 operator+(f3 a, f3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ f3 operator-(f3 a, f3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ f3 operator-(f3 a) { return {-a.x, -a.y, -a.z}; }
__device__ __forceinline__ f3 operator*(float s, f3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ f3 operator*(f3 a, float s) { return {a.x * s, a.y * s, a.z * s}; }
__device__ __forceinline__ f3 operator/(f3 a, float s) { return {a.x / s, a.y / s, a.z / s}; }
__device__ __forceinline__ f3 operator*(int s, f3 a) { return float(s) * a; }
__device__ __forceinline__ f3 operator*(f3 a, int s) { return a * float(s); }
__device__ __forceinline__ f3 operator/(f3 a, int s) { return a / float(s); }

// ---- matrix operators
__device__ __forceinline__ M3 operator+(M3 const &a, M3 const &b) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = a.m[k] + b.m[k];
  return r;
}
__device__ __forceinline__ M3 operator-(M3 const &a, M3 const &b) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = a.m[k] - b.m[k];
  return r;
}
__device__ __forceinline__ M3 operator-(M3 const &a) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = -a.m[k];
  return r;
}
__device__ __forceinline__ M3 operator*(float s, M3 const &a) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = s * a.m[k];
  return r;
}
__device__ __forceinline__ M3 operator*(M3 const &a, float s) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = a.m[k] * s;
  return r;
}
__device__ __forceinline__ M3 operator/(M3 const &a, float s) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = a.m[k] / s;
  return r;
}
// row . vector
__device__ __forceinline__ f3 operator*(M3 const &a, f3 v) {
  return {a.m[0] * v.x + (a.m[3] * v.y + a.m[6] * v.z), a.m[1] * v.x + (a.m[4] * v.y + a.m[7] * v.z),
          a.m[2] * v.x + (a.m[5] * v.y + a.m[8] * v.z)};
}
// row . column
__device__ __forceinline__ M3 operator*(M3 const &a, M3 const &b) {
  M3 r;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int i = 0; i < 3; ++i)
      r.m[3 * c + i] = a.m[i] * b.m[3 * c] + (a.m[3 + i] * b.m[3 * c + 1] + a.m[6 + i] * b.m[3 * c + 2]);
  return r;
}

// ---- compound assignment (Eigen's a op= b is a = a op b per component)
template <class A, class B> __device__ __forceinline__ void add_to(A &a, B const &b) { a = a + b; }
template <class A, class B> __device__ __forceinline__ void sub_from(A &a, B const &b) { a = a - b; }
template <class A, class B> __device__ __forceinline__ void mul_by(A &a, B const &b) { a = a * b; }
template <class A, class B> __device__ __forceinline__ void div_by(A &a, B const &b) { a = a / b; }

// ---- constants
template <class T> __device__ __forceinline__ T zeros();
template <> __device__ __forceinline__ float zeros<float>() { return 0.0f; }
template <> __device__ __forceinline__ int zeros<int>() { return 0; }
template <> __device__ __forceinline__ f3 zeros<f3>() { return {0.0f, 0.0f, 0.0f}; }
template <> __device__ __forceinline__ M3 zeros<M3>() {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = 0.0f;
  return r;
}
template <class T> __device__ __forceinline__ T ones();
template <> __device__ __forceinline__ float ones<float>() { return 1.0f; }
template <> __device__ __forceinline__ int ones<int>() { return 1; }
template <> __device__ __forceinline__ f3 ones<f3>() { return {1.0f, 1.0f, 1.0f}; }
template <> __device__ __forceinline__ M3 ones<M3>() {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = 1.0f;
  return r;
}
__device__ __forceinline__ M3 identity3() {
  M3 r = zeros<M3>();
  r.m[0] = r.m[4] = r.m[8] = 1.0f;
  return r;
}
template <class T> __device__ __forceinline__ T positive_infinity();
template <> __device__ __forceinline__ float positive_infinity<float>() { return __int_as_float(0x7f800000); }
template <class T> __device__ __forceinline__ T negative_infinity();
template <> __device__ __forceinline__ float negative_infinity<float>() { return __int_as_float(0xff800000); }

// ---- functions
__device__ __forceinline__ float dot(f3 a, f3 b) { return a.x * b.x + (a.y * b.y + a.z * b.z); }
__device__ __forceinline__ float norm_squared(float a) { return a * a; }
__device__ __forceinline__ float norm_squared(f3 a) { return dot(a, a); }
__device__ __forceinline__ float norm(float a) { return fabsf(a); }
__device__ __forceinline__ float norm(f3 a) { return sqrtf(norm_squared(a)); }
__device__ __forceinline__ float cabs(float a) { return fabsf(a); }
__device__ __forceinline__ f3 cabs(f3 a) { return {fabsf(a.x), fabsf(a.y), fabsf(a.z)}; }
__device__ __forceinline__ M3 cabs(M3 const &a) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = fabsf(a.m[k]);
  return r;
}
// std::max / std::min over an initializer list: the first largest (smallest)
template <class T> __device__ __forceinline__ T max(T a, T b) { return (a < b) ? b : a; }
template <class T, class... R> __device__ __forceinline__ T max(T a, T b, R... r) { return max(max(a, b), r...); }
template <class T> __device__ __forceinline__ T min(T a, T b) { return (b < a) ? b : a; }
template <class T, class... R> __device__ __forceinline__ T min(T a, T b, R... r) { return min(min(a, b), r...); }
__device__ __forceinline__ float reciprocal_or_zero(float x, float eps) { return (fabsf(x) > eps) ? 1.0f / x : 0.0f; }
template <class... R> __device__ __forceinline__ float unit_step_l(float eps, R... x) {
  return ((eps < x) || ...) ? 1.0f : 0.0f;
}
template <class... R> __device__ __forceinline__ float unit_step_r(float eps, R... x) {
  return ((eps <= x) || ...) ? 1.0f : 0.0f;
}
__device__ __forceinline__ M3 outer_product(f3 a, f3 b) {
  float av[3] = {a.x, a.y, a.z}, bv[3] = {b.x, b.y, b.z};
  M3 r;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int i = 0; i < 3; ++i) r.m[3 * c + i] = av[i] * bv[c];
  return r;
}
__device__ __forceinline__ M3 transpose(M3 const &a) {
  M3 r;
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int i = 0; i < 3; ++i) r.m[3 * c + i] = a.m[3 * i + c];
  return r;
}
__device__ __forceinline__ float trace(M3 const &a) { return a.m[0] + (a.m[4] + a.m[8]); }
__device__ __forceinline__ float invert(float a) { return 1.0f / a; }
__device__ __forceinline__ M3 invert(M3 const &a) { return minv3(a); }
__device__ __forceinline__ M3 invert_pm(M3 const &a) { return pinv3(a); }
__device__ __forceinline__ float smoothstep(float a) {
  float x = min(max(a, 0.0f), 1.0f);
  return (x * x) * (3.0f - 2.0f * x);
}
// Eigen's comma initializer fills row by row
__device__ __forceinline__ M3 cross_product_matrix_from_vector(f3 v) {
  M3 r;
  r.m[0] = 0.0f, r.m[3] = -v.z, r.m[6] = v.y;
  r.m[1] = v.z, r.m[4] = 0.0f, r.m[7] = -v.x;
  r.m[2] = -v.y, r.m[5] = v.x, r.m[8] = 0.0f;
  return r;
}
__device__ __forceinline__ f3 vector_from_cross_product_matrix(M3 const &a) { return {a.m[5], a.m[6], a.m[1]}; }

// components (slices): v[d]
__device__ __forceinline__ float &comp(f3 &v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }
__device__ __forceinline__ float comp(f3 const &v, int d) { return d == 0 ? v.x : (d == 1 ? v.y : v.z); }

// ---- the cubic spline kernel of the smoothing scale h
__device__ __forceinline__ float kernel_h(f3 v, float h) { return kW(kparams(h), v); }
__device__ __forceinline__ f3 kernel_gradient_h(f3 v, float h) { return kgradW(kparams(h), v); }
__device__ __forceinline__ float kernel_support_radius(float h) { return h * 2.0f; }

// ---- [AAT13] cohesion and adhesion splines (math/aat13.hpp); pow is
// CUDA's powf, so these agree with the reference's libm to a few ulp, not
// bit for bit
__device__ __forceinline__ float cpow2(float x) { return x * x; }
__device__ __forceinline__ float cpow3(float x) { return (x * x) * x; }
__device__ __forceinline__ float aat13_cohesion_h(float r, float h_diam) {
  float const pi = 3.14159265358979323846f;
  float h = 2.0f * h_diam;
  float h6 = powf(h, 6.0f), h9 = powf(h, 9.0f);
  float factor = 32.0f / (pi * h9);
  if (h < 2.0f * r && r <= h) return factor * (cpow3(h - r) * cpow3(r));
  if (0.0f <= r && 2.0f * r <= h) return factor * ((2.0f * cpow3(h - r)) * cpow3(r) - h6 / 64.0f);
  return 0.0f;
}
__device__ __forceinline__ float aat13_adhesion_h(float r, float h_diam) {
  float h = 2.0f * h_diam;
  float factor = 0.007f / powf(h, 3.25f);
  if (h < 2.0f * r && r <= h) {
    float b = ((-4.0f * cpow2(r)) / h + 6.0f * r) - 2.0f * h;
    return factor * powf(max(0.0f, b), 0.25f);
  }
  return 0.0f;
}

// ---- field storage
// varying: real -> float[n], real[] -> float4[n], real[][] -> 9 planes of
// cap floats (plane k = column-major index), integer -> int[n]
struct Planar9 {
  float *p;
  uint32_t cap;
};
__device__ __forceinline__ float rd(float const *a, uint32_t i) { return a[i]; }
__device__ __forceinline__ int rd(int const *a, uint32_t i) { return a[i]; }
__device__ __forceinline__ f3 rd(float4 const *a, uint32_t i) { return mk3(a[i]); }
__device__ __forceinline__ M3 rd(Planar9 a, uint32_t i) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = a.p[size_t(k) * a.cap + i];
  return r;
}
__device__ __forceinline__ void wr(float *a, uint32_t i, float v) { a[i] = v; }
__device__ __forceinline__ void wr(int *a, uint32_t i, int v) { a[i] = v; }
__device__ __forceinline__ void wr(float4 *a, uint32_t i, f3 v) { a[i] = make_float4(v.x, v.y, v.z, 0.0f); }
__device__ __forceinline__ void wr(Planar9 a, uint32_t i, M3 const &v) {
#pragma unroll
  for (int k = 0; k < 9; ++k) a.p[size_t(k) * a.cap + i] = v.m[k];
}
// uniform and global fields: the reference's host layout in the model's
// arena (components consecutive, matrices column-major)
struct SReal { float *p; };
struct SInt { int *p; };
struct SVec { float *p; };
struct SMat { float *p; };
__device__ __forceinline__ float rd(SReal s) { return *s.p; }
__device__ __forceinline__ int rd(SInt s) { return *s.p; }
__device__ __forceinline__ f3 rd(SVec s) { return {s.p[0], s.p[1], s.p[2]}; }
__device__ __forceinline__ M3 rd(SMat s) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = s.p[k];
  return r;
}
__device__ __forceinline__ void wr(SReal s, float v) { *s.p = v; }
__device__ __forceinline__ void wr(SInt s, int v) { *s.p = v; }
__device__ __forceinline__ void wr(SVec s, f3 v) { s.p[0] = v.x, s.p[1] = v.y, s.p[2] = v.z; }
__device__ __forceinline__ void wr(SMat s, M3 const &v) {
#pragma unroll
  for (int k = 0; k < 9; ++k) s.p[k] = v.m[k];
}

// procedure-level locals: 16-word slots of a device frame
template <class T> __device__ __forceinline__ T frd(float *fr, int slot);
template <> __device__ __forceinline__ float frd<float>(float *fr, int slot) { return fr[16 * slot]; }
template <> __device__ __forceinline__ int frd<int>(float *fr, int slot) { return __float_as_int(fr[16 * slot]); }
template <> __device__ __forceinline__ f3 frd<f3>(float *fr, int slot) {
  return {fr[16 * slot], fr[16 * slot + 1], fr[16 * slot + 2]};
}
template <> __device__ __forceinline__ M3 frd<M3>(float *fr, int slot) {
  M3 r;
#pragma unroll
  for (int k = 0; k < 9; ++k) r.m[k] = fr[16 * slot + k];
  return r;
}
__device__ __forceinline__ void fwr(float *fr, int slot, float v) { fr[16 * slot] = v; }
__device__ __forceinline__ void fwr(float *fr, int slot, int v) { fr[16 * slot] = __int_as_float(v); }
__device__ __forceinline__ void fwr(float *fr, int slot, f3 v) {
  fr[16 * slot] = v.x, fr[16 * slot + 1] = v.y, fr[16 * slot + 2] = v.z;
}
__device__ __forceinline__ void fwr(float *fr, int slot, M3 const &v) {
#pragma unroll
  for (int k = 0; k < 9; ++k) fr[16 * slot + k] = v.m[k];
}

// ---- reductions of a particle loop: per block, then in block order
__device__ __forceinline__ double block_reduce_max(double v, double *sh) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    double w = __shfl_down_sync(0xffffffffu, v, o);
    v = (v < w) ? w : v;
  }
  int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) sh[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int nw = (blockDim.x + 31) >> 5;
    v = (lane < nw) ? sh[lane] : -INFINITY;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      double w = __shfl_down_sync(0xffffffffu, v, o);
      v = (v < w) ? w : v;
    }
  }
  __syncthreads();
  return v;
}
__device__ __forceinline__ double block_reduce_min(double v, double *sh) { return -block_reduce_max(-v, sh); }

// ---- solve pcg: the generic preconditioned CG of the reference
// (solver/cg_openmp.hpp:35-215) over the particles of one group, values of
// type float (real) or f3 (real[], stored as float4).  The per-item dots
// are f32 (a0 b0 + (a1 b1 + a2 b2)); their sums, the threshold and the
// breaks are FP64 and alpha, beta the FP64 quotients rounded to f32, as the
// hand-written WKBB18 solver and the oracle's FP64 mode.
struct PcgState {
  double thr, r_nsq, prev_rdy, next_rdy, tol;
  float alpha, beta;
  int iter, stop, max_k;
};

__device__ __forceinline__ float vdot(float a, float b) { return a * b; }
__device__ __forceinline__ float vdot(f3 a, f3 b) { return dot(a, b); }
__device__ __forceinline__ float vld(float const *a, uint32_t i) { return a[i]; }
__device__ __forceinline__ f3 vld(float4 const *a, uint32_t i) { return mk3(a[i]); }
__device__ __forceinline__ void vst(float *a, uint32_t i, float v) { a[i] = v; }
__device__ __forceinline__ void vst(float4 *a, uint32_t i, f3 v) { a[i] = make_float4(v.x, v.y, v.z, 0.0f); }

constexpr int kPcgNT = 128;

__device__ __forceinline__ void pcg_commit(double v, double *part) {
  __shared__ double sh[32];
  double b = block_sum(v, sh);
  if (threadIdx.x == 0) part[blockIdx.x] = b;
}
// r = r - b; sum b.b
template <class S> __global__ void k_pcg_residual(uint32_t n, S *r, S const *b, double *part) {
  uint32_t i = blockIdx.x * kPcgNT + threadIdx.x;
  double v = 0.0;
  if (i < n) {
    auto bi = vld(b, i);
    vst(r, i, vld(r, i) - bi);
    v = double(vdot(bi, bi));
  }
  pcg_commit(v, part);
}
// p = -y; sums r.r and r.y
template <class S> __global__ void k_pcg_start(uint32_t n, S *p, S const *y, S const *r, double *part_rr,
                                               double *part_ry) {
  uint32_t i = blockIdx.x * kPcgNT + threadIdx.x;
  double rr = 0.0, ry = 0.0;
  if (i < n) {
    auto yi = vld(y, i), ri = vld(r, i);
    vst(p, i, -yi);
    rr = double(vdot(ri, ri));
    ry = double(vdot(ri, yi));
  }
  pcg_commit(rr, part_rr);
  pcg_commit(ry, part_ry);
}
// sum a.b
template <class S> __global__ void k_pcg_dot(uint32_t n, S const *a, S const *b, double *part) {
  uint32_t i = blockIdx.x * kPcgNT + threadIdx.x;
  double v = 0.0;
  if (i < n) v = double(vdot(vld(a, i), vld(b, i)));
  pcg_commit(v, part);
}
// x += alpha p; r += alpha q; sum r.r (nothing once the loop has stopped)
template <class S> __global__ void k_pcg_update(uint32_t n, S *x, S *r, S const *p, S const *q, PcgState const *st,
                                                double *part_rr) {
  uint32_t i = blockIdx.x * kPcgNT + threadIdx.x;
  double rr = 0.0;
  if (i < n && !st->stop) {
    float alpha = st->alpha;
    vst(x, i, vld(x, i) + alpha * vld(p, i));
    auto ri = vld(r, i) + alpha * vld(q, i);
    vst(r, i, ri);
    rr = double(vdot(ri, ri));
  }
  pcg_commit(rr, part_rr);
}
// p = -y + beta p
template <class S> __global__ void k_pcg_direction(uint32_t n, S *p, S const *y, PcgState const *st) {
  uint32_t i = blockIdx.x * kPcgNT + threadIdx.x;
  if (i < n && !st->stop) vst(p, i, -vld(y, i) + st->beta * vld(p, i));
}
__device__ __forceinline__ double pcg_sum(double const *part, uint32_t nb) {
  double a = 0.0;
  for (uint32_t b = 0; b < nb; ++b) a += part[b];
  return a;
}
__device__ __forceinline__ bool pcg_ok(PcgState const &s, int k, double r_nsq) {
  if (k < 1) return true;
  if (k > s.max_k) return false;
  return !(r_nsq < s.thr);
}
// after the initial residual and preconditioned iterate
__global__ void k_pcg_begin(PcgState *st, SReal tol, SInt max_k, double const *part_bb, double const *part_rr,
                            double const *part_ry, uint32_t nb) {
  PcgState s{};
  s.tol = double(rd(tol));
  s.max_k = rd(max_k);
  double b_nsq = pcg_sum(part_bb, nb);
  double thr = s.tol * s.tol * b_nsq;
  double fmin = double(1.17549435082228750797e-38f); // smallest positive normal f32
  s.thr = thr < fmin ? fmin : thr;
  s.r_nsq = pcg_sum(part_rr, nb);
  s.next_rdy = pcg_sum(part_ry, nb);
  s.iter = 0;
  s.stop = pcg_ok(s, 0, s.r_nsq) ? 0 : 1;
  *st = s;
}
// after q = A p: the first break test and alpha
__global__ void k_pcg_step(PcgState *st, double const *part_pq, uint32_t nb) {
  PcgState s = *st;
  if (s.stop) return;
  s.prev_rdy = s.next_rdy;
  double pdq = pcg_sum(part_pq, nb);
  if (fabs(pdq) < s.tol) {
    s.stop = 1;
  } else {
    s.alpha = float(s.prev_rdy / pdq);
  }
  *st = s;
}
// after y = T r: the second break test, beta, the iteration count and the
// loop condition
__global__ void k_pcg_next(PcgState *st, double const *part_rr, double const *part_ry, uint32_t nb) {
  PcgState s = *st;
  if (s.stop) return;
  s.r_nsq = pcg_sum(part_rr, nb);
  s.next_rdy = pcg_sum(part_ry, nb);
  if (fabs(s.prev_rdy) < s.tol) {
    s.stop = 1;
  } else {
    s.beta = float(s.next_rdy / s.prev_rdy);
    s.iter += 1;
    // the loop condition; the direction update is skipped once the loop is
    // over (the direction is not read after it)
    if (!pcg_ok(s, s.iter, s.r_nsq)) s.stop = 1;
  }
  *st = s;
}
__global__ void k_pcg_end(PcgState const *st, SInt iterations) { wr(iterations, st->iter); }
// an empty group: the solve returns 0 iterations
__global__ void k_pcg_zero(SInt iterations) { wr(iterations, 0); }

// the lists of a query group to neighbour group g
__device__ __forceinline__ NbrList nbr_list(NbrView const &v, int g) {
  return NbrList{v.chunks[g], v.idx32[g], v.cb[g], v.cap[g], v.n};
}

} // namespace dsl
} // namespace prtcl_gpu
