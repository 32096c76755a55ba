// 3x3 matrices of the schemes (real[3][3], column-major like the reference's
// Eigen matrices): inverse, pseudo-inverse and matrix-vector product, with
// the operation orders the oracle restates.  Shared by the hand-written
// schemes and by schemes generated from the scheme language.
#pragma once

#include "common.cuh"

namespace prtcl_gpu {

struct M3 {
  float m[9]; // column-major
};

__device__ __forceinline__ float cof3(M3 const &A, int i, int j) {
  int i1 = (i + 1) % 3, i2 = (i + 2) % 3, j1 = (j + 1) % 3, j2 = (j + 2) % 3;
  return A.m[3 * j1 + i1] * A.m[3 * j2 + i2] - A.m[3 * j2 + i1] * A.m[3 * j1 + i2];
}
// inverse by the adjugate (cofactors, determinant along column 0)
__device__ __forceinline__ M3 minv3(M3 const &A) {
  float c00 = cof3(A, 0, 0), c10 = cof3(A, 1, 0), c20 = cof3(A, 2, 0);
  float det = c00 * A.m[0] + (c10 * A.m[1] + c20 * A.m[2]);
  float inv = 1.0f / det;
  M3 r;
  r.m[0] = c00 * inv;           // (0,0)
  r.m[3] = c10 * inv;           // (0,1)
  r.m[6] = c20 * inv;           // (0,2)
  r.m[1] = cof3(A, 0, 1) * inv; // (1,0)
  r.m[4] = cof3(A, 1, 1) * inv; // (1,1)
  r.m[7] = cof3(A, 2, 1) * inv; // (1,2)
  r.m[2] = cof3(A, 0, 2) * inv; // (2,0)
  r.m[5] = cof3(A, 1, 2) * inv; // (2,1)
  r.m[8] = cof3(A, 2, 2) * inv; // (2,2)
  return r;
}

// Moore-Penrose pseudo-inverse of a 3x3 matrix: one-sided Jacobi SVD
// (Hestenes), 8 sweeps over the column pairs (0,1), (0,2), (1,2); A V = W
// with orthogonal columns w_i = sigma_i u_i, A+ = sum_i v_i w_i^T / sigma_i^2
// over the sigma_i > 3 eps sigma_max.  Stands in for the reference's
// invert_pm (math/impl/eigen.hpp:266-276, Eigen's complete orthogonal
// decomposition); the oracle runs the same operations.
__device__ __forceinline__ float dot3r(float const *a, float const *b) { return a[0] * b[0] + (a[1] * b[1] + a[2] * b[2]); }
__device__ inline M3 pinv3(M3 const &A) {
  float w[3][3], v[3][3];
#pragma unroll
  for (int c = 0; c < 3; ++c)
#pragma unroll
    for (int r = 0; r < 3; ++r) {
      w[c][r] = A.m[3 * c + r];
      v[c][r] = (r == c) ? 1.0f : 0.0f;
    }
  for (int sweep = 0; sweep < 8; ++sweep)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
      int p = k < 2 ? 0 : 1, q = k == 0 ? 1 : 2;
      float alpha = dot3r(w[p], w[p]), beta = dot3r(w[q], w[q]), gamma = dot3r(w[p], w[q]);
      if (gamma == 0.0f) continue;
      float zeta = (beta - alpha) / (2.0f * gamma);
      float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
      float c = 1.0f / sqrtf(1.0f + t * t);
      float sn = c * t;
#pragma unroll
      for (int r = 0; r < 3; ++r) {
        float wp = w[p][r], wq = w[q][r];
        w[p][r] = c * wp - sn * wq;
        w[q][r] = sn * wp + c * wq;
        float vp = v[p][r], vq = v[q][r];
        v[p][r] = c * vp - sn * vq;
        v[q][r] = sn * vp + c * vq;
      }
    }
  float s2[3], smax = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    s2[i] = dot3r(w[i], w[i]);
    float si = sqrtf(s2[i]);
    if (si > smax) smax = si;
  }
  float thr = 3.0f * 1.1920928955078125e-07f * smax;
  M3 R;
#pragma unroll
  for (int e = 0; e < 9; ++e) R.m[e] = 0.0f;
#pragma unroll
  for (int i = 0; i < 3; ++i) {
    if (!(sqrtf(s2[i]) > thr)) continue;
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
      for (int r = 0; r < 3; ++r) R.m[3 * c + r] = R.m[3 * c + r] + (v[i][r] * w[i][c]) / s2[i];
  }
  return R;
}

// L g for a column-major 3x3 L (row . vector, a0 + (a1 + a2))
__device__ __forceinline__ f3 mv3(float const (&L)[9], f3 g) {
  return {L[0] * g.x + (L[3] * g.y + L[6] * g.z), L[1] * g.x + (L[4] * g.y + L[7] * g.z),
          L[2] * g.x + (L[5] * g.y + L[8] * g.z)};
}

} // namespace prtcl_gpu
