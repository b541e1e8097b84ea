// Per-tet constitutive math for the sm_103a element kernel.
//
// Everything here runs in registers of one thread (one tet).  3x3 matrices are
// column major, a[i + 3*j] = A(i,j), matching the reference's flatten()
// (util/MATRIX_UTIL.cpp:33-43).  The deformation gradient, its SVD and the
// stress are FP64; the eigen-clamped Hessian is templated on the arithmetic
// type so the mixed-precision path can build it in FP32.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace hobak {

__device__ __forceinline__ double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[7] * A[5]) - A[3] * (A[1] * A[8] - A[7] * A[2]) +
         A[6] * (A[1] * A[5] - A[4] * A[2]);
}

// Sort A's (orthogonal) columns by norm, form U = A / sigma (completing
// vanishing columns), and fold reflections into S[2] (svd_rv convention).
__device__ __forceinline__ void svd3_finish(double* A, double* U, double* S, double* V) {
  double n[3];
#pragma unroll
  for (int k = 0; k < 3; k++) n[k] = A[3 * k] * A[3 * k] + A[3 * k + 1] * A[3 * k + 1] + A[3 * k + 2] * A[3 * k + 2];
  // sort columns by norm, descending (3-element network, swaps A and V columns)
  auto swapcols = [&](int a, int b) {
    double tn = n[a];
    n[a] = n[b];
    n[b] = tn;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double t = A[3 * a + i];
      A[3 * a + i] = A[3 * b + i];
      A[3 * b + i] = t;
      t = V[3 * a + i];
      V[3 * a + i] = V[3 * b + i];
      V[3 * b + i] = t;
    }
  };
  if (n[0] < n[1]) swapcols(0, 1);
  if (n[0] < n[2]) swapcols(0, 2);
  if (n[1] < n[2]) swapcols(1, 2);
  // sigma = sqrt(n) and 1/sigma from one reciprocal square root each
  double rs[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    rs[k] = n[k] > 0.0 ? rsqrt(n[k]) : 0.0;
    S[k] = n[k] * rs[k];
  }
  // U columns; complete vanishing columns with cross products
  const double tiny = 1e-300;
  if (S[0] > tiny) {
    const double r0 = rs[0];
#pragma unroll
    for (int i = 0; i < 3; i++) U[i] = A[i] * r0;
  } else {
    U[0] = 1.0; U[1] = 0.0; U[2] = 0.0;
  }
  if (S[1] > tiny) {
    const double r1 = rs[1];
#pragma unroll
    for (int i = 0; i < 3; i++) U[3 + i] = A[3 + i] * r1;
  } else {
    // unit vector orthogonal to u0: cross u0 with the axis it is least aligned with
    const double ax = fabs(U[0]), ay = fabs(U[1]), az = fabs(U[2]);
    double e0 = 0, e1 = 0, e2 = 0;
    if (ax <= ay && ax <= az) e0 = 1; else if (ay <= az) e1 = 1; else e2 = 1;
    double w0 = U[1] * e2 - U[2] * e1, w1 = U[2] * e0 - U[0] * e2, w2 = U[0] * e1 - U[1] * e0;
    const double rn = rsqrt(w0 * w0 + w1 * w1 + w2 * w2);
    U[3] = w0 * rn; U[4] = w1 * rn; U[5] = w2 * rn;
  }
  if (S[2] > tiny && S[1] > tiny) {
    const double r2 = rs[2];
#pragma unroll
    for (int i = 0; i < 3; i++) U[6 + i] = A[6 + i] * r2;
  } else {
    U[6] = U[1] * U[5] - U[2] * U[4];
    U[7] = U[2] * U[3] - U[0] * U[5];
    U[8] = U[0] * U[4] - U[1] * U[3];
  }
  if (det3(U) < 0.0) {
    U[6] = -U[6]; U[7] = -U[7]; U[8] = -U[8];
    S[2] = -S[2];
  }
  if (det3(V) < 0.0) {
    V[6] = -V[6]; V[7] = -V[7]; V[8] = -V[8];
    S[2] = -S[2];
  }
}

// Rotation-variant SVD F = U diag(S) V^T (the svd_rv convention,
// util/MATRIX_UTIL.cpp:76-95): S sorted by magnitude, U and V rotations, the
// sign of det F carried by S[2].  One-sided Jacobi: plane rotations applied
// on the right orthogonalise F's columns; V accumulates them.  Converges
// quadratically; the loop stops when no pair needs a rotation.
__device__ __forceinline__ void svd3_rv(const double* F, double* U, double* S, double* V) {
  double A[9];
#pragma unroll
  for (int k = 0; k < 9; k++) A[k] = F[k];
#pragma unroll
  for (int k = 0; k < 9; k++) V[k] = (k % 4 == 0) ? 1.0 : 0.0;
  for (int sweep = 0; sweep < 12; sweep++) {
    bool rotated = false;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const int p = (r == 2) ? 1 : 0;
      const int q = (r == 0) ? 1 : 2;
      const double alpha = A[3 * p] * A[3 * p] + A[3 * p + 1] * A[3 * p + 1] + A[3 * p + 2] * A[3 * p + 2];
      const double beta = A[3 * q] * A[3 * q] + A[3 * q + 1] * A[3 * q + 1] + A[3 * q + 2] * A[3 * q + 2];
      const double gamma = A[3 * p] * A[3 * q] + A[3 * p + 1] * A[3 * q + 1] + A[3 * p + 2] * A[3 * q + 2];
      if (gamma * gamma > 1e-30 * (alpha * beta)) {  // off-diagonal above ~1e-15 relative
        rotated = true;
        const double zeta = (beta - alpha) / (2.0 * gamma);
        const double t = copysign(1.0, zeta) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
        const double c = rsqrt(1.0 + t * t), s = c * t;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double x = A[3 * p + i], y = A[3 * q + i];
          A[3 * p + i] = c * x - s * y;
          A[3 * q + i] = s * x + c * y;
          const double vx = V[3 * p + i], vy = V[3 * q + i];
          V[3 * p + i] = c * vx - s * vy;
          V[3 * q + i] = s * vx + c * vy;
        }
      }
    }
    if (!rotated) break;
  }
  svd3_finish(A, U, S, V);
}

// The same SVD with most of the Jacobi work moved off the FP64 pipe, which is
// the scarce resource on GB300 (FP32 issues far faster):
//   1. one-sided Jacobi sweeps in FP32 give V32 with F V32 orthogonal to
//      ~3e-7 (a few FP32 ulps; more FP32 sweeps cost far less than an FP64 one);
//   2. V32 is re-orthonormalised in FP64 (modified Gram-Schmidt), so V stays an
//      exact rotation to FP64 precision;
//   3. FP64 one-sided Jacobi on A = F V finishes the job; starting ~3e-7 from
//      orthogonal, one sweep brings well-separated columns to ~1e-13
//      (quadratic convergence) and the second sweep only checks; nearly
//      equal singular values may take one more rotating sweep.  Rotation
//      angles are computed in FP32 and turned into an exactly orthogonal
//      (c, s) pair in FP64.
// V is a rotation to FP64 rounding and F = U S V^T holds to FP64 rounding;
// U's columns are orthogonal to 1e-12 relative (the stop test), which keeps
// forces and Hessians within ~1e-12 of a fully converged SVD while sparing
// rotating sweeps of ~110 FP64 instructions per element each.
__device__ __forceinline__ void svd3_rv_fast(const double* F, double* U, double* S, double* V) {
  // ---- stage 1: FP32 Jacobi ----
  float a[9], w[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    a[k] = float(F[k]);
    w[k] = (k % 4 == 0) ? 1.0f : 0.0f;
  }
  for (int sweep = 0; sweep < 10; sweep++) {
    bool rotated = false;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const int p = (r == 2) ? 1 : 0;
      const int q = (r == 0) ? 1 : 2;
      const float al = a[3 * p] * a[3 * p] + a[3 * p + 1] * a[3 * p + 1] + a[3 * p + 2] * a[3 * p + 2];
      const float be = a[3 * q] * a[3 * q] + a[3 * q + 1] * a[3 * q + 1] + a[3 * q + 2] * a[3 * q + 2];
      const float ga = a[3 * p] * a[3 * q] + a[3 * p + 1] * a[3 * q + 1] + a[3 * p + 2] * a[3 * q + 2];
      if (fabsf(ga) > 3e-7f * sqrtf(al * be)) {  // a few FP32 ulps above the rounding noise
        rotated = true;
        const float zeta = (be - al) / (2.0f * ga);
        const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
        const float c = rsqrtf(1.0f + t * t), s = c * t;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const float x = a[3 * p + i], y = a[3 * q + i];
          a[3 * p + i] = c * x - s * y;
          a[3 * q + i] = s * x + c * y;
          const float vx = w[3 * p + i], vy = w[3 * q + i];
          w[3 * p + i] = c * vx - s * vy;
          w[3 * q + i] = s * vx + c * vy;
        }
      }
    }
    if (!rotated) break;
  }
  // ---- stage 2: FP64 modified Gram-Schmidt on V32's columns ----
#pragma unroll
  for (int k = 0; k < 3; k++) {
#pragma unroll
    for (int i = 0; i < 3; i++) V[3 * k + i] = double(w[3 * k + i]);
#pragma unroll
    for (int j = 0; j < k; j++) {
      const double d = V[3 * j] * V[3 * k] + V[3 * j + 1] * V[3 * k + 1] + V[3 * j + 2] * V[3 * k + 2];
#pragma unroll
      for (int i = 0; i < 3; i++) V[3 * k + i] -= d * V[3 * j + i];
    }
    const double n = rsqrt(V[3 * k] * V[3 * k] + V[3 * k + 1] * V[3 * k + 1] + V[3 * k + 2] * V[3 * k + 2]);
#pragma unroll
    for (int i = 0; i < 3; i++) V[3 * k + i] *= n;
  }
  // ---- stage 3: FP64 Jacobi on A = F V ----
  double A[9];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++) A[i + 3 * j] = F[i] * V[3 * j] + F[i + 3] * V[3 * j + 1] + F[i + 6] * V[3 * j + 2];
  for (int sweep = 0; sweep < 8; sweep++) {
    bool rotated = false;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const int p = (r == 2) ? 1 : 0;
      const int q = (r == 0) ? 1 : 2;
      const double alpha = A[3 * p] * A[3 * p] + A[3 * p + 1] * A[3 * p + 1] + A[3 * p + 2] * A[3 * p + 2];
      const double beta = A[3 * q] * A[3 * q] + A[3 * q + 1] * A[3 * q + 1] + A[3 * q + 2] * A[3 * q + 2];
      const double gamma = A[3 * p] * A[3 * q] + A[3 * p + 1] * A[3 * q + 1] + A[3 * p + 2] * A[3 * q + 2];
      if (gamma * gamma > 1e-24 * (alpha * beta)) {  // columns orthogonal to 1e-12 relative
        rotated = true;
        // angle in FP32 (only orthogonality of (c, s) must be FP64-exact)
        const float zf = float(beta - alpha) / (2.0f * float(gamma));
        const float tf = copysignf(1.0f, zf) / (fabsf(zf) + sqrtf(1.0f + zf * zf));
        const double t = double(tf);
        const double c = rsqrt(1.0 + t * t), s = c * t;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double x = A[3 * p + i], y = A[3 * q + i];
          A[3 * p + i] = c * x - s * y;
          A[3 * q + i] = s * x + c * y;
          const double vx = V[3 * p + i], vy = V[3 * q + i];
          V[3 * p + i] = c * vx - s * vy;
          V[3 * q + i] = s * vx + c * vy;
        }
      }
    }
    if (!rotated) break;
  }
  svd3_finish(A, U, S, V);
}

// The rotation-variant SVD in FP32 alone (stage 1 of svd3_rv_fast, then the
// svd3_finish steps in FP32): for the mixed-precision path of the energies
// whose stress needs no SVD (SNH, STVK, LINEAR, NEO_HOOKEAN_BW,
// SNH_WITH_BARRIER: their PK1 is a function of F), where the factors only
// feed the FP32 eigen-clamped Hessian.  The same svd_rv convention: S sorted
// by magnitude, U and V rotations, a reflection carried by the sign of S[2].
__device__ __forceinline__ void svd3_rv_f32(const double* F, float* U, float* S, float* V) {
  float a[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    a[k] = float(F[k]);
    V[k] = (k % 4 == 0) ? 1.0f : 0.0f;
  }
  for (int sweep = 0; sweep < 10; sweep++) {
    bool rotated = false;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const int p = (r == 2) ? 1 : 0;
      const int q = (r == 0) ? 1 : 2;
      const float al = a[3 * p] * a[3 * p] + a[3 * p + 1] * a[3 * p + 1] + a[3 * p + 2] * a[3 * p + 2];
      const float be = a[3 * q] * a[3 * q] + a[3 * q + 1] * a[3 * q + 1] + a[3 * q + 2] * a[3 * q + 2];
      const float ga = a[3 * p] * a[3 * q] + a[3 * p + 1] * a[3 * q + 1] + a[3 * p + 2] * a[3 * q + 2];
      if (fabsf(ga) > 3e-7f * sqrtf(al * be)) {
        rotated = true;
        const float zeta = (be - al) / (2.0f * ga);
        const float t = copysignf(1.0f, zeta) / (fabsf(zeta) + sqrtf(1.0f + zeta * zeta));
        const float c = rsqrtf(1.0f + t * t), s = c * t;
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const float x = a[3 * p + i], y = a[3 * q + i];
          a[3 * p + i] = c * x - s * y;
          a[3 * q + i] = s * x + c * y;
          const float vx = V[3 * p + i], vy = V[3 * q + i];
          V[3 * p + i] = c * vx - s * vy;
          V[3 * q + i] = s * vx + c * vy;
        }
      }
    }
    if (!rotated) break;
  }
  // sort columns by norm, descending
  float n[3];
#pragma unroll
  for (int k = 0; k < 3; k++) n[k] = a[3 * k] * a[3 * k] + a[3 * k + 1] * a[3 * k + 1] + a[3 * k + 2] * a[3 * k + 2];
  auto swapcols = [&](int x, int y) {
    float tn = n[x];
    n[x] = n[y];
    n[y] = tn;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      float t = a[3 * x + i];
      a[3 * x + i] = a[3 * y + i];
      a[3 * y + i] = t;
      t = V[3 * x + i];
      V[3 * x + i] = V[3 * y + i];
      V[3 * y + i] = t;
    }
  };
  if (n[0] < n[1]) swapcols(0, 1);
  if (n[0] < n[2]) swapcols(0, 2);
  if (n[1] < n[2]) swapcols(1, 2);
  float rs[3];
#pragma unroll
  for (int k = 0; k < 3; k++) {
    rs[k] = n[k] > 0.0f ? rsqrtf(n[k]) : 0.0f;
    S[k] = n[k] * rs[k];
  }
  const float tiny = 1e-30f;
  if (S[0] > tiny) {
#pragma unroll
    for (int i = 0; i < 3; i++) U[i] = a[i] * rs[0];
  } else {
    U[0] = 1.0f; U[1] = 0.0f; U[2] = 0.0f;
  }
  if (S[1] > tiny) {
#pragma unroll
    for (int i = 0; i < 3; i++) U[3 + i] = a[3 + i] * rs[1];
  } else {
    const float ax = fabsf(U[0]), ay = fabsf(U[1]), az = fabsf(U[2]);
    float e0 = 0, e1 = 0, e2 = 0;
    if (ax <= ay && ax <= az) e0 = 1; else if (ay <= az) e1 = 1; else e2 = 1;
    const float w0 = U[1] * e2 - U[2] * e1, w1 = U[2] * e0 - U[0] * e2, w2 = U[0] * e1 - U[1] * e0;
    const float rn = rsqrtf(w0 * w0 + w1 * w1 + w2 * w2);
    U[3] = w0 * rn; U[4] = w1 * rn; U[5] = w2 * rn;
  }
  if (S[2] > tiny && S[1] > tiny) {
#pragma unroll
    for (int i = 0; i < 3; i++) U[6 + i] = a[6 + i] * rs[2];
  } else {
    U[6] = U[1] * U[5] - U[2] * U[4];
    U[7] = U[2] * U[3] - U[0] * U[5];
    U[8] = U[0] * U[4] - U[1] * U[3];
  }
  auto det = [](const float* A) {
    return A[0] * (A[4] * A[8] - A[7] * A[5]) - A[3] * (A[1] * A[8] - A[7] * A[2]) +
           A[6] * (A[1] * A[5] - A[4] * A[2]);
  };
  if (det(U) < 0.0f) {
    U[6] = -U[6]; U[7] = -U[7]; U[8] = -U[8];
    S[2] = -S[2];
  }
  if (det(V) < 0.0f) {
    V[6] = -V[6]; V[7] = -V[7]; V[8] = -V[8];
    S[2] = -S[2];
  }
}

// ARAP's rotation R = U V^T (the rotation of F's polar decomposition in the
// svd_rv convention) in FP64 from the FP32 factors of svd3_rv_f32:
//   1. R0 = U V^T, re-orthonormalised in FP64 (Gram-Schmidt of two columns,
//      the third their cross product, so det R0 = +1);
//   2. one correction R = R0 Q, Q = I + W + W^2 / 2 with W = [w]x, where w
//      solves (tr(S) I - S) w = (Y32 - Y23, Y13 - Y31, Y21 - Y12) for
//      Y = R0^T F and S = sym(Y): the rotation that makes Q^T Y symmetric.
// From R0 within ~1e-7 of R the result is within ~1e-14 while tr(S) I - S
// (eigenvalues sigma_i + sigma_j) is well conditioned.  Returns false when
// sigma_1 + sigma_2 is below 1e-2 sigma_0 (near ARAP's twist singularity, or
// a collapsed tet): the caller then takes the FP64 SVD.
__device__ __forceinline__ bool arap_rotation_refined(const double* F, const float* U, const float* S, const float* V,
                                                      double* R) {
  if (!(S[1] + S[2] > 1e-2f * S[0])) return false;
  double c0[3], c1[3];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    c0[i] = double(U[i] * V[0] + U[i + 3] * V[3] + U[i + 6] * V[6]);
    c1[i] = double(U[i] * V[1] + U[i + 3] * V[4] + U[i + 6] * V[7]);
  }
  const double n0 = rsqrt(c0[0] * c0[0] + c0[1] * c0[1] + c0[2] * c0[2]);
#pragma unroll
  for (int i = 0; i < 3; i++) c0[i] *= n0;
  const double d01 = c0[0] * c1[0] + c0[1] * c1[1] + c0[2] * c1[2];
#pragma unroll
  for (int i = 0; i < 3; i++) c1[i] -= d01 * c0[i];
  const double n1 = rsqrt(c1[0] * c1[0] + c1[1] * c1[1] + c1[2] * c1[2]);
#pragma unroll
  for (int i = 0; i < 3; i++) c1[i] *= n1;
  double R0[9];
#pragma unroll
  for (int i = 0; i < 3; i++) {
    R0[i] = c0[i];
    R0[3 + i] = c1[i];
  }
  R0[6] = c0[1] * c1[2] - c0[2] * c1[1];
  R0[7] = c0[2] * c1[0] - c0[0] * c1[2];
  R0[8] = c0[0] * c1[1] - c0[1] * c1[0];
  // Y = R0^T F
  double Y[9];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++)
      Y[i + 3 * j] = R0[3 * i] * F[3 * j] + R0[3 * i + 1] * F[3 * j + 1] + R0[3 * i + 2] * F[3 * j + 2];
  // K = tr(S) I - S, S = sym(Y); rhs = twice the axial vector of skew(Y)
  const double tr = Y[0] + Y[4] + Y[8];
  const double k00 = tr - Y[0], k11 = tr - Y[4], k22 = tr - Y[8];
  const double k01 = -0.5 * (Y[3] + Y[1]), k02 = -0.5 * (Y[6] + Y[2]), k12 = -0.5 * (Y[7] + Y[5]);
  const double b0 = Y[5] - Y[7], b1 = Y[6] - Y[2], b2 = Y[1] - Y[3];
  // w = K^-1 b by cofactors (K symmetric)
  const double a00 = k11 * k22 - k12 * k12, a01 = k02 * k12 - k01 * k22, a02 = k01 * k12 - k02 * k11;
  const double a11 = k00 * k22 - k02 * k02, a12 = k01 * k02 - k00 * k12, a22 = k00 * k11 - k01 * k01;
  const double det = k00 * a00 + k01 * a01 + k02 * a02;
  const double id = 1.0 / det;
  const double w0 = id * (a00 * b0 + a01 * b1 + a02 * b2);
  const double w1 = id * (a01 * b0 + a11 * b1 + a12 * b2);
  const double w2 = id * (a02 * b0 + a12 * b1 + a22 * b2);
  // R = R0 (I + W + W^2 / 2), W^2 = w w^T - |w|^2 I
  const double h = 1.0 - 0.5 * (w0 * w0 + w1 * w1 + w2 * w2);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double r0 = R0[i], r1 = R0[i + 3], r2 = R0[i + 6];
    const double rw = 0.5 * (r0 * w0 + r1 * w1 + r2 * w2);
    // row i of R0 W: (r1 w2 - r2 w1, r2 w0 - r0 w2, r0 w1 - r1 w0)
    R[i] = h * r0 + (r1 * w2 - r2 * w1) + rw * w0;
    R[i + 3] = h * r1 + (r2 * w0 - r0 * w2) + rw * w1;
    R[i + 6] = h * r2 + (r0 * w1 - r1 * w0) + rw * w2;
  }
  return true;
}

// Symmetric 3x3 eigensystem by cyclic Jacobi: A = Q diag(L) Q^T.
template <typename T>
__device__ __forceinline__ void eig3sym(const T* Ain, T* Q, T* L) {
  T a00 = Ain[0], a01 = Ain[3], a02 = Ain[6], a11 = Ain[4], a12 = Ain[7], a22 = Ain[8];
#pragma unroll
  for (int k = 0; k < 9; k++) Q[k] = (k % 4 == 0) ? T(1) : T(0);
  const T eps = sizeof(T) == 8 ? T(1e-15) : T(1e-6);  // just above each type's rounding floor
  for (int sweep = 0; sweep < 16; sweep++) {
    const T off = fabs(a01) + fabs(a02) + fabs(a12);
    const T dg = fabs(a00) + fabs(a11) + fabs(a22);
    if (!(off > eps * dg)) break;
#pragma unroll
    for (int r = 0; r < 3; r++) {
      const int p = (r == 2) ? 1 : 0;
      const int q = (r == 0) ? 1 : 2;
      T apq = (r == 0) ? a01 : (r == 1) ? a02 : a12;
      if (apq == T(0)) continue;
      T app = (p == 0) ? a00 : a11;
      T aqq = (q == 1) ? a11 : a22;
      const T theta = (aqq - app) / (T(2) * apq);
      const T t = copysign(T(1), theta) / (fabs(theta) + sqrt(theta * theta + T(1)));
      const T c = T(1) / sqrt(t * t + T(1)), s = t * c;
      // rotate: the remaining index m is the third one
      if (r == 0) {  // (0,1), m = 2
        const T n00 = a00 - t * a01, n11 = a11 + t * a01;
        const T n02 = c * a02 - s * a12, n12 = s * a02 + c * a12;
        a00 = n00; a11 = n11; a01 = T(0); a02 = n02; a12 = n12;
      } else if (r == 1) {  // (0,2), m = 1
        const T n00 = a00 - t * a02, n22 = a22 + t * a02;
        const T n01 = c * a01 - s * a12, n21 = s * a01 + c * a12;
        a00 = n00; a22 = n22; a02 = T(0); a01 = n01; a12 = n21;
      } else {  // (1,2), m = 0
        const T n11 = a11 - t * a12, n22 = a22 + t * a12;
        const T n01 = c * a01 - s * a02, n02 = s * a01 + c * a02;
        a11 = n11; a22 = n22; a12 = T(0); a01 = n01; a02 = n02;
      }
#pragma unroll
      for (int m = 0; m < 3; m++) {
        const T qp = Q[m + 3 * p], qq = Q[m + 3 * q];
        Q[m + 3 * p] = c * qp - s * qq;
        Q[m + 3 * q] = s * qp + c * qq;
      }
    }
  }
  L[0] = a00; L[1] = a11; L[2] = a22;
}

// Material parameters after each reference constructor's reparameterisation.
struct MatParams {
  int kind;
  double mu, lambda, alpha;
  double a[3];  // anisotropic energies: unit fibre direction
};

// fiber: the anisotropic energies' direction, normalised here as their
// constructors do (ANISOTROPIC_ARAP.cpp:26-29); ignored by the isotropic ones.
__host__ __device__ inline MatParams make_material(int kind, double mu, double lambda,
                                                   const double* fiber = nullptr) {
  MatParams m{kind, mu, lambda, 0.0, {1.0, 0.0, 0.0}};
  if (fiber) {
    const double n = sqrt(fiber[0] * fiber[0] + fiber[1] * fiber[1] + fiber[2] * fiber[2]);
    for (int i = 0; i < 3; i++) m.a[i] = n > 0.0 ? fiber[i] / n : fiber[i];
  }
  if (kind == MAT_SNH) {  // SNH.cpp:23-32
    m.lambda = lambda + mu;
    m.alpha = 1.0 + m.mu / m.lambda;
  } else if (kind == MAT_NHBW) {  // NEO_HOOKEAN_BW.cpp:23-29
    m.alpha = 1.0 + mu / lambda;
  } else if (kind == MAT_SNHB) {  // SNH_WITH_BARRIER.cpp:26-35
    m.mu = (4.0 / 3.0) * mu;
    m.lambda = lambda + (5.0 / 6.0) * mu;
    m.alpha = 1.0 + m.mu / m.lambda - m.mu / (4.0 * m.lambda);
  }
  return m;
}

// d det(F) / dF = [f1 x f2, f2 x f0, f0 x f1] (partialJpartialF, MATRIX_UTIL.cpp:561-568)
__device__ __forceinline__ void cofactor(const double* F, double* G) {
  G[0] = F[4] * F[8] - F[5] * F[7];
  G[1] = F[5] * F[6] - F[3] * F[8];
  G[2] = F[3] * F[7] - F[4] * F[6];
  G[3] = F[7] * F[2] - F[8] * F[1];
  G[4] = F[8] * F[0] - F[6] * F[2];
  G[5] = F[6] * F[1] - F[7] * F[0];
  G[6] = F[1] * F[5] - F[2] * F[4];
  G[7] = F[2] * F[3] - F[0] * F[5];
  G[8] = F[0] * F[4] - F[1] * F[3];
}

// psi(F): SNH.cpp:34-43, ARAP.cpp:39-43, STVK.cpp psi, LINEAR.cpp psi,
// NEO_HOOKEAN_BW.cpp psi, SNH_WITH_BARRIER.cpp psi.  ARAP uses the SVD given.
__device__ inline double material_psi(const MatParams& m, const double* F, const double* S) {
  double Ic = 0;
#pragma unroll
  for (int k = 0; k < 9; k++) Ic += F[k] * F[k];
  switch (m.kind) {
    case MAT_SNH: {
      const double Jm = det3(F) - m.alpha;
      return 0.5 * (m.mu * (Ic - 3.0) + m.lambda * Jm * Jm);
    }
    case MAT_ARAP:
      return m.mu * ((S[0] - 1.0) * (S[0] - 1.0) + (S[1] - 1.0) * (S[1] - 1.0) + (S[2] - 1.0) * (S[2] - 1.0));
    case MAT_STVK: {
      double E[9], tr = 0, en = 0;
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double ftf = F[3 * i] * F[3 * j] + F[3 * i + 1] * F[3 * j + 1] + F[3 * i + 2] * F[3 * j + 2];
          E[i + 3 * j] = 0.5 * (ftf - (i == j ? 1.0 : 0.0));
        }
      tr = E[0] + E[4] + E[8];
#pragma unroll
      for (int k = 0; k < 9; k++) en += E[k] * E[k];
      return m.mu * en + m.lambda * 0.5 * tr * tr;
    }
    case MAT_LINEAR: {
      double en = 0;
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double e = 0.5 * (F[i + 3 * j] + F[j + 3 * i]) - (i == j ? 1.0 : 0.0);
          en += e * e;
        }
      const double tr = F[0] + F[4] + F[8] - 3.0;
      return m.mu * en + 0.5 * m.lambda * tr * tr;
    }
    case MAT_NHBW: {
      const double lj = log(det3(F));
      return m.mu * 0.5 * (Ic - 3.0) - m.mu * lj + m.lambda * 0.5 * lj * lj;
    }
    default: {  // MAT_SNHB
      const double Jm = det3(F) - m.alpha;
      return 0.5 * (m.mu * (Ic - 3.0) + m.lambda * Jm * Jm - m.mu * log(Ic + 1.0));
    }
  }
}

// PK1(F): SNH.cpp:45-50, ARAP.cpp:48-55 (P = R 2mu (S - I) = 2mu (F - U V^T)),
// STVK.cpp PK1, LINEAR.cpp PK1, NEO_HOOKEAN_BW.cpp PK1, SNH_WITH_BARRIER.cpp PK1.
__device__ inline void material_pk1_of_F(const MatParams& m, const double* F, double* P);

__device__ inline void material_pk1(const MatParams& m, const double* F, const double* U, const double* V,
                                    double* P) {
  if (m.kind == MAT_ARAP) {
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const double R = U[i] * V[j] + U[i + 3] * V[j + 3] + U[i + 6] * V[j + 6];
        P[i + 3 * j] = 2.0 * m.mu * (F[i + 3 * j] - R);
      }
    return;
  }
  material_pk1_of_F(m, F, P);
}

// PK1 of the energies whose stress is a function of F alone (every isotropic
// energy but ARAP).
__device__ inline void material_pk1_of_F(const MatParams& m, const double* F, double* P) {
  switch (m.kind) {
    case MAT_SNH: {
      double G[9];
      cofactor(F, G);
      const double s = m.lambda * (det3(F) - m.alpha);
#pragma unroll
      for (int k = 0; k < 9; k++) P[k] = m.mu * F[k] + s * G[k];
      return;
    }
    case MAT_STVK: {
      double E[9];
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double ftf = F[3 * i] * F[3 * j] + F[3 * i + 1] * F[3 * j + 1] + F[3 * i + 2] * F[3 * j + 2];
          E[i + 3 * j] = 0.5 * (ftf - (i == j ? 1.0 : 0.0));
        }
      const double tr = E[0] + E[4] + E[8];
      double Sg[9];
#pragma unroll
      for (int k = 0; k < 9; k++) Sg[k] = (k % 4 == 0 ? m.lambda * tr : 0.0) + 2.0 * m.mu * E[k];
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++)
          P[i + 3 * j] = F[i] * Sg[3 * j] + F[i + 3] * Sg[3 * j + 1] + F[i + 6] * Sg[3 * j + 2];
      return;
    }
    case MAT_LINEAR: {
      const double tr = F[0] + F[4] + F[8] - 3.0;
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) {
          const double e = 0.5 * (F[i + 3 * j] + F[j + 3 * i]) - (i == j ? 1.0 : 0.0);
          P[i + 3 * j] = 2.0 * m.mu * e + (i == j ? m.lambda * tr : 0.0);
        }
      return;
    }
    case MAT_NHBW: {
      double G[9];
      cofactor(F, G);
      const double J = det3(F), iJ = 1.0 / J, lj = log(J);
#pragma unroll
      for (int k = 0; k < 9; k++) P[k] = m.mu * (F[k] - iJ * G[k]) + m.lambda * lj * iJ * G[k];
      return;
    }
    default: {  // MAT_SNHB
      double G[9], Ic = 0;
      cofactor(F, G);
#pragma unroll
      for (int k = 0; k < 9; k++) Ic += F[k] * F[k];
      const double s = m.lambda * (det3(F) - m.alpha), b = m.mu / (Ic + 1.0);
#pragma unroll
      for (int k = 0; k < 9; k++) P[k] = m.mu * F[k] + s * G[k] - b * F[k];
      return;
    }
  }
}

// Analytic eigensystem of the 9x9 Hessian d2psi/dF2 in the (twist, flip,
// scaling) basis of "Analytic Eigensystems for Isotropic Distortion Energies":
// L[0..2] twist, L[3..5] flip, L[6..8] scaling with 3x3 scaling-mode matrix A
// (symmetric, column major).  Returns false when the scaling modes are the
// coordinate axes (ARAP, MATRIX_UTIL.cpp:465-497 "jackpot" version).
// SNH.cpp:94-144, ARAP.cpp:113-135, STVK.cpp buildEigensystem,
// NEO_HOOKEAN_BW.cpp clampedHessian, SNH_WITH_BARRIER.cpp clampedHessian.
template <typename T, typename IT = double>
__device__ inline bool material_eigensystem(const MatParams& mp, const IT* Sd, T* L, T* A) {
  const T mu = T(mp.mu), lambda = T(mp.lambda);
  const T s0 = T(Sd[0]), s1 = T(Sd[1]), s2 = T(Sd[2]);
  switch (mp.kind) {
    case MAT_ARAP: {
      L[0] = mu * (T(2) - T(4) / (s1 + s2));
      L[1] = mu * (T(2) - T(4) / (s0 + s2));
      L[2] = mu * (T(2) - T(4) / (s0 + s1));
#pragma unroll
      for (int k = 3; k < 9; k++) L[k] = T(2) * mu;
      return false;
    }
    case MAT_SNH: {
      const T J = s0 * s1 * s2;
      const T front = lambda * (J - T(1)) - mu;
      L[0] = front * s0 + mu;
      L[1] = front * s1 + mu;
      L[2] = front * s2 + mu;
      L[3] = -front * s0 + mu;
      L[4] = -front * s1 + mu;
      L[5] = -front * s2 + mu;
      A[0] = mu + lambda * s1 * s1 * s2 * s2;
      A[4] = mu + lambda * s0 * s0 * s2 * s2;
      A[8] = mu + lambda * s0 * s0 * s1 * s1;
      const T od = lambda * (T(2) * J - T(1)) - mu;
      A[1] = A[3] = od * s2;
      A[2] = A[6] = od * s1;
      A[5] = A[7] = od * s0;
      return true;
    }
    case MAT_STVK: {
      const T I2 = s0 * s0 + s1 * s1 + s2 * s2;
      const T front = -mu + lambda * T(0.5) * (I2 - T(3));
      L[0] = front + mu * (s1 * s1 + s2 * s2 - s1 * s2);
      L[1] = front + mu * (s0 * s0 + s2 * s2 - s0 * s2);
      L[2] = front + mu * (s0 * s0 + s1 * s1 - s0 * s1);
      L[3] = front + mu * (s1 * s1 + s2 * s2 + s1 * s2);
      L[4] = front + mu * (s0 * s0 + s2 * s2 + s0 * s2);
      L[5] = front + mu * (s0 * s0 + s1 * s1 + s0 * s1);
      const T sv[3] = {s0, s1, s2};
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++)
          A[i + 3 * j] = (i == j) ? front + (lambda + T(3) * mu) * sv[i] * sv[i] : lambda * sv[i] * sv[j];
      return true;
    }
    case MAT_NHBW: {
      const T J = s0 * s1 * s2, lj = log(J);
      const T i01 = T(1) / (s0 * s1), i02 = T(1) / (s0 * s2), i12 = T(1) / (s1 * s2);
      const T front = lambda * lj - mu;
      L[0] = front * i12 + mu;
      L[1] = front * i02 + mu;
      L[2] = front * i01 + mu;
      L[3] = -front * i12 + mu;
      L[4] = -front * i02 + mu;
      L[5] = -front * i01 + mu;
      const T fd = lambda * (T(1) - lj) + mu;
      A[0] = fd / (s0 * s0) + mu;
      A[4] = fd / (s1 * s1) + mu;
      A[8] = fd / (s2 * s2) + mu;
      A[1] = A[3] = lambda * i01;
      A[2] = A[6] = lambda * i02;
      A[5] = A[7] = lambda * i12;
      return true;
    }
    default: {  // MAT_SNHB
      const T alpha = T(mp.alpha);
      const T J = s0 * s1 * s2, I2 = s0 * s0 + s1 * s1 + s2 * s2;
      const T front = -mu / (I2 + T(1)) + mu;
      const T back = lambda * (J - alpha);
      L[0] = front + back * s0;
      L[1] = front + back * s1;
      L[2] = front + back * s2;
      L[3] = front - back * s0;
      L[4] = front - back * s1;
      L[5] = front - back * s2;
      const T isq = T(1) / ((I2 + T(1)) * (I2 + T(1))), tm = T(2) * mu;
      const T fd = (-mu * (I2 + T(1))) * isq + mu;
      const T fo = (T(2) * J - alpha) * lambda;
      A[0] = fd + tm * s0 * s0 * isq + lambda * s1 * s1 * s2 * s2;
      A[4] = fd + tm * s1 * s1 * isq + lambda * s0 * s0 * s2 * s2;
      A[8] = fd + tm * s2 * s2 * isq + lambda * s0 * s0 * s1 * s1;
      A[1] = A[3] = fo * s2 + (tm * s0 * s1) * isq;
      A[2] = A[6] = fo * s1 + (tm * s0 * s2) * isq;
      A[5] = A[7] = fo * s0 + (tm * s1 * s2) * isq;
      return true;
    }
  }
}

// ---- anisotropic energies (Hyperelastic/Volume/ANISOTROPIC_*.cpp) ----
// With the unit fibre direction a, g = F a, F A = g a^T (A = a a^T) and
// I5 = |g|^2 (invariant5, MATRIX_UTIL.cpp:553-556), every stress is a scalar
// times F A and every Hessian is alpha H5 + beta vec(FA) vec(FA)^T with
// H5 = kronIdentity(A) (MATRIX_UTIL.cpp:512-524).  Pushed through pFpx, that
// Hessian is the Kronecker product (c c^T) (x) (alpha I + beta g g^T) with
// c = (-sum d, d) and d = DmInv a: a 3x3 block per vertex pair, no 9x9 form.

// I4 = a^T (V Sigma V^T) a from the svd_rv factors (invariant4,
// MATRIX_UTIL.cpp:545-552); ANISOTROPIC_ARAP reads its sign and |I4| < 1e-8.
__device__ __forceinline__ double aniso_invariant4(const MatParams& m, const double* S, const double* V) {
  double I4 = 0.0;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double va = V[3 * k] * m.a[0] + V[3 * k + 1] * m.a[1] + V[3 * k + 2] * m.a[2];
    I4 += S[k] * va * va;
  }
  return I4;
}

// g = F a and I5 = |g|^2
__device__ __forceinline__ double aniso_stretch(const MatParams& m, const double* F, double* g) {
#pragma unroll
  for (int i = 0; i < 3; i++) g[i] = F[i] * m.a[0] + F[i + 3] * m.a[1] + F[i + 6] * m.a[2];
  return g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
}

// psi: ANISOTROPIC_ARAP.cpp:40-47, ANISOTROPIC_STVK.cpp:42-46,
// ANISOTROPIC_FUNG.cpp:40-44, ANISOTROPIC_DIRICHLET.cpp:36-39
__device__ inline double aniso_psi(const MatParams& m, double I5, double I4) {
  switch (m.kind) {
    case MAT_AARAP: {
      const double d = sqrt(I5) - (I4 > 0.0 ? 1.0 : -1.0);
      return 0.5 * m.mu * d * d;
    }
    case MAT_ASTVK: return 0.5 * m.mu * (I5 - 1.0) * (I5 - 1.0);
    case MAT_AFUNG: return m.mu * (exp(I5 - 1.0) - I5);
    default: return m.mu * I5;
  }
}

// s with P = s F A: ANISOTROPIC_ARAP.cpp:52-65 (near I4 = 0 the reference's
// fixed value), ANISOTROPIC_STVK.cpp:51-55, ANISOTROPIC_FUNG.cpp:50-54,
// ANISOTROPIC_DIRICHLET.cpp:44-47
__device__ inline double aniso_pk1_scale(const MatParams& m, double I5, double I4) {
  switch (m.kind) {
    case MAT_AARAP:
      return fabs(I4) >= 1e-8 ? m.mu * (1.0 - (I4 > 0.0 ? 1.0 : -1.0) / sqrt(I5)) : -0.5 * m.mu;
    case MAT_ASTVK: return 2.0 * m.mu * (I5 - 1.0);
    case MAT_AFUNG: return 2.0 * m.mu * (exp(I5 - 1.0) - 1.0);
    default: return 2.0 * m.mu;
  }
}

// (alpha, beta) of the Hessian alpha H5 + beta fa fa^T, unclamped (hessian)
// or clamped (clampedHessian): ANISOTROPIC_ARAP.cpp:70-110,
// ANISOTROPIC_STVK.cpp:60-100, ANISOTROPIC_FUNG.cpp:60-105,
// ANISOTROPIC_DIRICHLET.cpp:52-77.  fa2 = |vec(F A)|^2 (= I5 for a unit a).
__device__ inline void aniso_hessian_coeffs(const MatParams& m, double I5, double I4, double fa2, bool clamp,
                                            double& al, double& be) {
  if (m.kind == MAT_AARAP) {
    const double SI4 = I4 > 0.0 ? 1.0 : -1.0;
    if (!clamp || I5 >= SI4) {
      const double si = 1.0 / sqrt(I5);
      al = m.mu * (1.0 - SI4 * si);
      be = m.mu * (SI4 * si * si * si);
    } else {
      al = 0.0;
      be = m.mu * (1.0 / I5);
    }
    return;
  }
  if (m.kind == MAT_ADIR) {
    al = 2.0 * m.mu;
    be = 0.0;
    return;
  }
  const bool fung = m.kind == MAT_AFUNG;
  const double e = fung ? exp(I5 - 1.0) : 1.0;
  const double l1 = fung ? 2.0 * m.mu * (e - 1.0) : 2.0 * m.mu * (I5 - 1.0);
  const double l0 = fung ? l1 + 4.0 * m.mu * I5 * e : l1 + 4.0 * m.mu * I5;
  if (!clamp || (l0 > 0.0 && l1 > 0.0)) {
    al = l1;
    be = 4.0 * m.mu * e;
  } else if (l0 < 0.0) {
    al = be = 0.0;
  } else {  // the rank-one part along fa / |fa| only (fa itself when |fa| = 0)
    al = 0.0;
    be = fa2 > 0.0 ? l0 / fa2 : l0;
  }
}

// 9x9 (column major, flatten order) alpha H5 + beta fa fa^T of F
__device__ inline void aniso_hessian9(const MatParams& m, const double* F, double I4, bool clamp, double* H) {
  double g[3];
  const double I5 = aniso_stretch(m, F, g);
  const double a2 = m.a[0] * m.a[0] + m.a[1] * m.a[1] + m.a[2] * m.a[2];
  double al, be;
  aniso_hessian_coeffs(m, I5, I4, I5 * a2, clamp, al, be);
  for (int c = 0; c < 9; c++)
    for (int r = 0; r < 9; r++) {
      const double h5 = (r % 3 == c % 3) ? m.a[r / 3] * m.a[c / 3] : 0.0;
      H[r + 9 * c] = al * h5 + be * (g[r % 3] * m.a[r / 3]) * (g[c % 3] * m.a[c / 3]);
    }
}

}  // namespace hobak
