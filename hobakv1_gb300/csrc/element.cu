// Per-tet element kernels for sm_103a.
//
// One thread per tet: gather the 4 vertices, F = Ds DmInv, rotation-variant
// SVD, PK1 and the analytic-eigensystem clamped Hessian, then the element
// force and the 12x12 element Hessian.  The Hessian is never formed as 9x9:
// every eigenmode q_k (a 3x3 matrix U M_k V^T) is pushed through
// pFpx^T first, w_k = pFpx^T vec(q_k), which only needs B = DmInv V, and the
// element matrix is accumulated as -vol D^T (sum_k lambda_k w_k w_k^T) D with
// D the 9x12 difference operator dx_a = x_{a+1} - x_0.  This is the same
// matrix as the reference's pFpx^T (-V clampedHessian) pFpx
// (TET_MESH_FASTER.cpp:95-103) with far fewer FP64 operations.
#include "element_math.cuh"
#include "kernels.cuh"

namespace hobak {

namespace {

constexpr double kInvSqrt2 = 0.70710678118654752440;

// 9x9 symmetric accumulator over (vertex a = 1..3, component i), packed
// upper triangle, index of (r, c) with r <= c.
__host__ __device__ __forceinline__ constexpr int sym9(int r, int c) { return r * 9 - (r * (r - 1)) / 2 + (c - r); }

// Hr = sum_k L_k w_k w_k^T over the 9 eigenmodes (reduced 9x9, vertices 1..3).
// Returns in Hr[45].  U, B are the SVD's U and B = DmInv V.
// clamp = false keeps negative eigenvalues: the unclamped hessian()
// (HYPERELASTIC.h:44) from the same eigensystem.
template <typename T, typename IT = double>
__device__ __forceinline__ void reduced_hessian(const MatParams& m, const IT* Ud, const IT* Sd, const IT* Vd,
                                                const double* Dinv, T* Hr, bool clamp = true) {
#pragma unroll
  for (int k = 0; k < 45; k++) Hr[k] = T(0);
  if (m.kind == MAT_LINEAR) {
    // H9 = mu (I + transpose swap) + lambda vec(I) vec(I)^T (LINEAR.cpp hessian):
    // Hr[(a,i),(b,k)] = mu delta_ik (d_a . d_b) + mu d_a[k] d_b[i] + lambda d_a[i] d_b[k]
    const T mu = T(m.mu), la = T(m.lambda);
#pragma unroll
    for (int r = 0; r < 9; r++)
#pragma unroll
      for (int c = r; c < 9; c++) {
        const int a = r / 3, i = r % 3, b = c / 3, k = c % 3;
        T dd = T(0);
#pragma unroll
        for (int j = 0; j < 3; j++) dd += T(Dinv[a + 3 * j]) * T(Dinv[b + 3 * j]);
        T val = mu * T(Dinv[a + 3 * k]) * T(Dinv[b + 3 * i]) + la * T(Dinv[a + 3 * i]) * T(Dinv[b + 3 * k]);
        if (i == k) val += mu * dd;
        Hr[sym9(r, c)] = val;
      }
    return;
  }
  T L[9], A3[9], Q3[9];
  const bool scalingMatrix = material_eigensystem<T, IT>(m, Sd, L, A3);
  if (scalingMatrix) {
    T L3[3];
    eig3sym<T>(A3, Q3, L3);
    L[6] = L3[0];
    L[7] = L3[1];
    L[8] = L3[2];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) Q3[k] = (k % 4 == 0) ? T(1) : T(0);
  }
  // B(a, m) = sum_j DmInv(a, j) V(j, m), computed in T; U in T
  T U[9], B[9], Dt[9], Vt[9];
#pragma unroll
  for (int k = 0; k < 9; k++) {
    U[k] = T(Ud[k]);
    Dt[k] = T(Dinv[k]);
    Vt[k] = T(Vd[k]);
  }
#pragma unroll
  for (int mm = 0; mm < 3; mm++)
#pragma unroll
    for (int a = 0; a < 3; a++) {
      T s = T(0);
#pragma unroll
      for (int j = 0; j < 3; j++) s += Dt[a + 3 * j] * Vt[j + 3 * mm];
      B[a + 3 * mm] = s;
    }
  const T rs2 = T(kInvSqrt2);
#pragma unroll
  for (int k = 0; k < 9; k++) {
    const T lam = (!clamp || L[k] > T(0)) ? L[k] : T(0);  // clamp (SNH.cpp:138-141)
    if (lam == T(0)) continue;
    T w[9];  // w[(a, comp)] = (U M_k B^T)(comp, a)
    if (k < 6) {
      // twist (k < 3) and flip (k >= 3) for column pair (i, j)
      const int kk = k % 3;
      const int i = (kk == 0) ? 1 : (kk == 1) ? 2 : 1;
      const int j = (kk == 0) ? 2 : 0;
      const T sgn = (k < 3) ? T(-1) : T(1);
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++)
          w[3 * a + c] = rs2 * (U[c + 3 * j] * B[a + 3 * i] + sgn * U[c + 3 * i] * B[a + 3 * j]);
    } else {
      const int kk = k - 6;
#pragma unroll
      for (int a = 0; a < 3; a++)
#pragma unroll
        for (int c = 0; c < 3; c++) {
          T s = T(0);
#pragma unroll
          for (int mm = 0; mm < 3; mm++) s += Q3[mm + 3 * kk] * U[c + 3 * mm] * B[a + 3 * mm];
          w[3 * a + c] = s;
        }
    }
#pragma unroll
    for (int r = 0; r < 9; r++) {
      const T lr = lam * w[r];
#pragma unroll
      for (int c = r; c < 9; c++) Hr[sym9(r, c)] += lr * w[c];
    }
  }
}

// Element force f = -vol pFpx^T vec(P) (TET_MESH.cpp:743-745):
// f_{a+1} = -vol P DmInv^T(:, a), f_0 = -(f_1 + f_2 + f_3).
__device__ __forceinline__ void element_force(const double* P, const double* Dinv, double vol, double* f) {
#pragma unroll
  for (int i = 0; i < 3; i++) f[i] = 0.0;
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double g = P[i] * Dinv[a] + P[i + 3] * Dinv[a + 3] + P[i + 6] * Dinv[a + 6];
      f[3 * (a + 1) + i] = -vol * g;
      f[i] += vol * g;
    }
}

// Expand -vol D^T Hr D into the 10 upper 3x3 blocks (row major in each block).
template <typename T, typename OutT>
__device__ __forceinline__ void expand_blocks(const T* Hr, double vol, OutT* out) {
  const T nv = T(-vol);
  // vertex-0 sums: colsum[b][i][k] = sum_a Hr[(a,i),(b,k)]
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int b = a; b < 3; b++)
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const int r = 3 * a + i, c = 3 * b + k;
          const T h = (r <= c) ? Hr[sym9(r, c)] : Hr[sym9(c, r)];
          out[9 * upper_block(a + 1, b + 1) + 3 * i + k] = OutT(nv * h);
        }
  T s00[9];
#pragma unroll
  for (int k = 0; k < 9; k++) s00[k] = T(0);
#pragma unroll
  for (int b = 0; b < 3; b++)
#pragma unroll
    for (int i = 0; i < 3; i++)
#pragma unroll
      for (int k = 0; k < 3; k++) {
        T s = T(0);
#pragma unroll
        for (int a = 0; a < 3; a++) {
          const int r = 3 * a + i, c = 3 * b + k;
          s += (r <= c) ? Hr[sym9(r, c)] : Hr[sym9(c, r)];
        }
        // block (0, b+1) entry (i, k) = -vol * (-(sum_a Hr[(a,i),(b,k)]))
        out[9 * upper_block(0, b + 1) + 3 * i + k] = OutT(-nv * s);
        s00[3 * i + k] += s;
      }
  // block (0,0) = -vol * sum_a sum_b Hr[a,b]: row sums of the column sums
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) out[3 * i + k] = OutT(nv * s00[3 * i + k]);
}

// The same 10 blocks as expand_blocks, with the same sums in the same order,
// emitted in memory order two values per store (8-byte stores for FP32,
// 16-byte for FP64): 45 store instructions per tet instead of 90, which
// relieves the load/store queue the per-tet kernels saturate.  out is the
// tet's record, 16-byte aligned so that the assembly reads each block with
// 16-byte loads: 92 values per tet, the last two padding written as zeros.
template <typename T, typename OutT>
__device__ __forceinline__ void store_blocks(const T* Hr, double vol, OutT* out) {
  const T nv = T(-vol);
  auto h = [&](int r, int c) -> T { return r <= c ? Hr[sym9(r, c)] : Hr[sym9(c, r)]; };
  auto value = [&](int e) -> OutT {
    const int ub = e / 9, i = (e % 9) / 3, k = e % 3;
    const int A = ub < 4 ? 0 : ub < 7 ? 1 : ub < 9 ? 2 : 3;
    const int B = ub < 4 ? ub : ub < 7 ? ub - 3 : ub < 9 ? ub - 5 : 3;
    if (A >= 1) return OutT(nv * h(3 * (A - 1) + i, 3 * (B - 1) + k));
    if (B >= 1) {
      T s = T(0);
#pragma unroll
      for (int a = 0; a < 3; a++) s += h(3 * a + i, 3 * (B - 1) + k);
      return OutT(-nv * s);
    }
    T s00 = T(0);
#pragma unroll
    for (int b = 0; b < 3; b++) {
      T s = T(0);
#pragma unroll
      for (int a = 0; a < 3; a++) s += h(3 * a + i, 3 * b + k);
      s00 += s;
    }
    return OutT(nv * s00);
  };
#pragma unroll
  for (int e = 0; e < kElemHess; e += 2) {
    if (sizeof(OutT) == 4) {
      *reinterpret_cast<float2*>(out + e) = make_float2(float(value(e)), float(value(e + 1)));
    } else {
      *reinterpret_cast<double2*>(out + e) = make_double2(double(value(e)), double(value(e + 1)));
    }
  }
  // the padding too: a partly written sector costs a DRAM read on eviction
  if (sizeof(OutT) == 4)
    *reinterpret_cast<float2*>(out + kElemHess) = make_float2(0.f, 0.f);
  else
    *reinterpret_cast<double2*>(out + kElemHess) = make_double2(0.0, 0.0);
}

// 12 doubles (16-byte aligned) as six 16-byte stores
__device__ __forceinline__ void store12(double* dst, const double* v) {
#pragma unroll
  for (int k = 0; k < 12; k += 2) *reinterpret_cast<double2*>(dst + k) = make_double2(v[k], v[k + 1]);
}

__device__ __forceinline__ void load_tet(const int4 tv, const double* rest, const double* x, double X[4][3]) {
  const int vid[4] = {tv.x, tv.y, tv.z, tv.w};
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) X[a][i] = rest[3 * vid[a] + i] + x[3 * vid[a] + i];
}

__device__ __forceinline__ void deformation_gradient(const double X[4][3], const double* Dinv, double* F) {
  // F = Ds DmInv, Ds(:, a) = x_{a+1} - x_0 (TET_MESH.cpp:706-714)
  double Ds[9];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) Ds[i + 3 * a] = X[a + 1][i] - X[0][i];
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++)
      F[i + 3 * j] = Ds[i] * Dinv[3 * j] + Ds[i + 3] * Dinv[1 + 3 * j] + Ds[i + 6] * Dinv[2 + 3 * j];
}

// Which tets an instantiation of k_element evaluates: every isotropic tet
// (the FP64 path), or, in the mixed path, split by whether the stress reads
// the SVD.  The other isotropic energies' PK1 is a function of F, so their
// SVD only feeds the FP32 Hessian and runs in FP32 (svd3_rv_f32); ARAP's
// PK1 = 2 mu (F - U V^T) reads the rotation in FP64, refined from the FP32
// factors (arap_rotation_refined), or from the FP64 SVD where that
// refinement is ill-conditioned.
constexpr int kElemAll = 0, kElemSvdFree = 1, kElemArap = 2;

// Batched step kernel: element Hessian blocks and right-hand-side terms
// g = dt (f + dt He v) for every tet of every scene.
// HT is the Hessian's arithmetic/storage type: double (FP64 path) or float
// (mixed path: F, stress and forces stay FP64; the SVD is FP64 where the
// stress reads it).
// Whether an instantiation evaluates tets of a scene of this kind.
template <int KC>
__device__ __forceinline__ bool evaluates(int kind) {
  if (is_anisotropic(kind)) return false;  // k_element_aniso
  return KC == kElemAll || (KC == kElemSvdFree) == (kind != MAT_ARAP);
}

template <typename HT, int KC>
// FP32 Hessians fit 128 registers (4 CTAs per SM); the FP64 variant needs
// ~208 and spills heavily below that.
__global__ void __launch_bounds__(128, sizeof(HT) == 4 ? 4 : 1)
    k_element(DeviceBatch b, int rawForces, HT* __restrict__ outH) {
  // The CTA's tets read their corners from shared memory: the distinct
  // vertices of its one or two staging blocks (host-built, ascending ids)
  // are loaded once each, rest + x and v, so each vertex position is summed
  // and fetched once per CTA instead of once per tet corner.
  extern __shared__ double stage[];  // [n][6]: rest + x, v
  const int tFirst = blockIdx.x * blockDim.x;
  const int tLast = min(b.nt, tFirst + (int)blockDim.x) - 1;
  // CTAs holding only scenes this instantiation does not evaluate (scenes
  // are contiguous in tet order) leave before staging
  {
    bool any = false;
    for (int sc = b.tetScene[tFirst]; sc <= b.tetScene[tLast] && !any; sc++) any = evaluates<KC>(b.scenes[sc].kind);
    if (!any) return;
  }
  const int sb0 = tFirst / kStageTets;
  const int s0 = b.stagePtr[sb0], s1 = b.stagePtr[tLast / kStageTets + 1];
  for (int i = threadIdx.x; i < s1 - s0; i += blockDim.x) {
    const int vid = b.stageVerts[s0 + i];
#pragma unroll
    for (int k = 0; k < 3; k++) {
      stage[6 * i + k] = b.rest[3 * vid + k] + b.x[3 * vid + k];
      stage[6 * i + 3 + k] = b.v[3 * vid + k];
    }
  }
  __syncthreads();
  const int t = tFirst + threadIdx.x;
  if (t > tLast) return;
  const SceneParams& sp = b.scenes[b.tetScene[t]];
  if (!sp.active || !evaluates<KC>(sp.kind)) return;
  // Newmark: a scene whose Newton loop is over needs no further element terms
  if (!rawForces && sp.integrator == kIntegratorNewmark && b.solve[b.tetScene[t]].newtonDone) return;
  const uchar4 lc = b.stageLocal[t];
  const int off = b.stagePtr[t / kStageTets] - s0;
  const double* sx[4] = {stage + 6 * (off + lc.x), stage + 6 * (off + lc.y), stage + 6 * (off + lc.z),
                         stage + 6 * (off + lc.w)};
  const MatParams m{sp.kind, sp.mu, sp.lambda, sp.alpha};
  // rhs term: dt (f + dt He v) for BACKWARD_EULER_VELOCITY; the force itself
  // for BACKWARD_EULER_POSITION (its rhs has no K v term: the Rayleigh part
  // uses the rest-state Hessian, k_rhs) and for raw forces (inspection)
  const bool velocityTerm = !rawForces && sp.integrator == kIntegratorVelocity;
  const double dt = velocityTerm ? sp.dt : 0.0;
  double Dinv[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Dinv[k] = b.DmInv[9 * (size_t)t + k];
  const double vol = b.vol[t];
  double X[4][3];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) X[a][i] = sx[a][i];
  double F[9], P[9], f[12];
  deformation_gradient(X, Dinv, F);
  HT Hr[45];
  if (KC == kElemSvdFree) {
    float U[9], S[3], V[9];
    svd3_rv_f32(F, U, S, V);
    material_pk1_of_F(m, F, P);
    // dt f directly (the force scaled by dt * vol instead of vol)
    element_force(P, Dinv, velocityTerm ? dt * vol : vol, f);
    reduced_hessian<HT, float>(m, U, S, V, Dinv, Hr);
  } else if (KC == kElemArap) {
    // the FP32 factors feed the FP32 Hessian; the stress's rotation is
    // refined to FP64 from them (the FP64 SVD near the twist singularity)
    float U[9], S[3], V[9];
    svd3_rv_f32(F, U, S, V);
    double R[9];
    if (!arap_rotation_refined(F, U, S, V, R)) {
      double Ud[9], Sd[3], Vd[9];
      svd3_rv_fast(F, Ud, Sd, Vd);
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) R[i + 3 * j] = Ud[i] * Vd[j] + Ud[i + 3] * Vd[j + 3] + Ud[i + 6] * Vd[j + 6];
    }
    // P = 2 mu (F - R) (ARAP.cpp:48-55)
#pragma unroll
    for (int k = 0; k < 9; k++) P[k] = 2.0 * m.mu * (F[k] - R[k]);
    element_force(P, Dinv, velocityTerm ? dt * vol : vol, f);
    reduced_hessian<HT, float>(m, U, S, V, Dinv, Hr);
  } else {
    double U[9], S[3], V[9];
    svd3_rv_fast(F, U, S, V);
    material_pk1(m, F, U, V, P);
    element_force(P, Dinv, velocityTerm ? dt * vol : vol, f);
    reduced_hessian<HT, double>(m, U, S, V, Dinv, Hr);
  }

  double* g = b.elemG + 12 * (size_t)t;
  if (!velocityTerm) {
    store12(g, f);
    store_blocks<HT, HT>(Hr, vol, outH + kElemHessStride * (size_t)t);
    return;
  }
  // He v = -vol D^T Hr (D v): D v = relative velocities of vertices 1..3
  // (in the mixed path He v is formed in FP32 like He itself)
  HT dv[9];
#pragma unroll
  for (int a = 0; a < 3; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) dv[3 * a + i] = HT(sx[a + 1][3 + i] - sx[0][3 + i]);
  // g = dt f + dt^2 He v: the He v rows carry the factor -vol dt^2 in HT
  // (one conversion and one add per entry on the FP64 pipe)
  const HT ch = HT(-vol * dt * dt);
  HT h0[3] = {HT(0), HT(0), HT(0)};
  double gl[12];
#pragma unroll
  for (int r = 0; r < 9; r++) {
    HT s = HT(0);
#pragma unroll
    for (int c = 0; c < 9; c++) s += ((r <= c) ? Hr[sym9(r, c)] : Hr[sym9(c, r)]) * dv[c];
    s *= ch;
    h0[r % 3] += s;
    gl[3 + r] = f[3 + r] + double(s);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) gl[i] = f[i] - double(h0[i]);
  store12(g, gl);
  store_blocks<HT, HT>(Hr, vol, outH + kElemHessStride * (size_t)t);
}

// Element terms of the anisotropic energies (ANISOTROPIC_ARAP, STVK, FUNG,
// DIRICHLET): P = s F A gives the element force f_{a+1} = -vol s g d_a,
// f_0 = vol s g (d_1 + d_2 + d_3) with g = F a and d = DmInv a, and the
// clamped Hessian alpha H5 + beta fa fa^T gives the element Hessian
// -vol (c c^T) (x) G with c = (-(d_1 + d_2 + d_3), d_1, d_2, d_3) and
// G = alpha I + beta g g^T: one 3x3 matrix per tet instead of a 9x9
// eigen-reconstruction.  Only ANISOTROPIC_ARAP needs the SVD (the sign of
// I4).  Same outputs, layout and precision split as k_element; launched
// beside it when the batch holds anisotropic scenes, so the isotropic
// kernel's code and registers are unchanged.
template <typename HT>
__global__ void __launch_bounds__(128) k_element_aniso(DeviceBatch b, int rawForces, HT* __restrict__ outH) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nt) return;
  const int sc = b.tetScene[t];
  const SceneParams& sp = b.scenes[sc];
  if (!sp.active || !is_anisotropic(sp.kind)) return;
  if (!rawForces && sp.integrator == kIntegratorNewmark && b.solve[sc].newtonDone) return;
  const int4 tv = b.tets[t];
  const MatParams m = make_material(sp.kind, sp.mu, sp.lambda, sp.fiber);
  const bool velocityTerm = !rawForces && sp.integrator == kIntegratorVelocity;
  const double dt = velocityTerm ? sp.dt : 0.0;
  double Dinv[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Dinv[k] = b.DmInv[9 * (size_t)t + k];
  const double vol = b.vol[t];
  double X[4][3], F[9], g[3];
  load_tet(tv, b.rest, b.x, X);
  deformation_gradient(X, Dinv, F);
  const double I5 = aniso_stretch(m, F, g);
  double I4 = 1.0;
  if (m.kind == MAT_AARAP) {
    double U[9], S[3], V[9];
    svd3_rv_fast(F, U, S, V);
    I4 = aniso_invariant4(m, S, V);
  }
  // d = DmInv a, c = (-(d1 + d2 + d3), d1, d2, d3)
  double c[4];
#pragma unroll
  for (int a = 0; a < 3; a++) c[a + 1] = Dinv[a] * m.a[0] + Dinv[a + 3] * m.a[1] + Dinv[a + 6] * m.a[2];
  c[0] = -(c[1] + c[2] + c[3]);
  const double fs = -(velocityTerm ? dt * vol : vol) * aniso_pk1_scale(m, I5, I4);
  double f[12];
#pragma unroll
  for (int a = 0; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) f[3 * a + i] = fs * c[a] * g[i];
  double al, be;
  const double a2 = m.a[0] * m.a[0] + m.a[1] * m.a[1] + m.a[2] * m.a[2];
  aniso_hessian_coeffs(m, I5, I4, I5 * a2, true, al, be);
  HT G[9];
#pragma unroll
  for (int i = 0; i < 3; i++)
#pragma unroll
    for (int k = 0; k < 3; k++) G[3 * i + k] = HT((i == k ? al : 0.0) + be * g[i] * g[k]);
  HT* out = outH + kElemHessStride * (size_t)t;
  const HT nv = HT(-vol);
#pragma unroll
  for (int A = 0; A < 4; A++)
#pragma unroll
    for (int B = A; B < 4; B++) {
      const HT cc = nv * HT(c[A]) * HT(c[B]);
#pragma unroll
      for (int e = 0; e < 9; e++) out[9 * upper_block(A, B) + e] = cc * G[e];
    }
  out[kElemHess] = HT(0);
  out[kElemHess + 1] = HT(0);
  double* gout = b.elemG + 12 * (size_t)t;
  if (!velocityTerm) {
#pragma unroll
    for (int k = 0; k < 12; k++) gout[k] = f[k];
    return;
  }
  // He v = -vol c_A G (sum_B c_B v_B), sum_B c_B v_B = sum_a d_a (v_a - v_0)
  const int vid[4] = {tv.x, tv.y, tv.z, tv.w};
  HT w[3] = {HT(0), HT(0), HT(0)};
#pragma unroll
  for (int a = 1; a < 4; a++)
#pragma unroll
    for (int i = 0; i < 3; i++) w[i] += HT(c[a]) * HT(b.v[3 * vid[a] + i] - b.v[3 * vid[0] + i]);
  const HT ch = HT(-vol * dt * dt);
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const HT gw = ch * (G[3 * i] * w[0] + G[3 * i + 1] * w[1] + G[3 * i + 2] * w[2]);
#pragma unroll
    for (int a = 0; a < 4; a++) gout[3 * a + i] = f[3 * a + i] + double(HT(c[a]) * gw);
  }
}

// 9x9 (column major, flatten order) of the reduced Hessian with DmInv = I:
// then Hr[(a,i),(b,k)] = H9[i + 3a, k + 3b].
__device__ __forceinline__ void reduced_to_h9(const double* Hr, double* H) {
#pragma unroll
  for (int r = 0; r < 9; r++)
#pragma unroll
    for (int c = 0; c < 9; c++) H[r + 9 * c] = (r <= c) ? Hr[sym9(r, c)] : Hr[sym9(c, r)];
}

// NEWMARK's energy-damped solve (NEWMARK.cpp:344-420): the GREEN_DAMPING
// force of every tet of a damped scene added to its element force, so the
// right-hand side's R holds the elastic and damping forces
// (TET_MESH::computeInternalForces).  The damping Hessian is passed to
// computeCollisionResponse, which zeroes it (TIMESTEPPER.cpp:657), so the
// system matrix is unchanged.  Per tet: the iterate's velocity
// S (a3 (x - x_old) + a4 v_old + a5 a_old) of its four vertices (zero at
// pins), Fdot = Vs DmInv (TET_MESH::computeFdots, TET_MESH.cpp:660-684),
// P = mu F (F^T Fdot + Fdot^T F) (GREEN_DAMPING.cpp:46-50) and the force
// -vol pFpx^T vec(P).  Runs after k_element, only in batches with a damped
// scene, so the element kernel itself is unchanged.
__global__ void __launch_bounds__(128) k_green_damping(DeviceBatch b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nt) return;
  const int sc = b.tetScene[t];
  const SceneParams& sp = b.scenes[sc];
  if (!sp.active || !(sp.greenMu > 0.0) || b.solve[sc].newtonDone) return;
  const int4 tv = b.tets[t];
  const int vid[4] = {tv.x, tv.y, tv.z, tv.w};
  double Dinv[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Dinv[k] = b.DmInv[9 * (size_t)t + k];
  double X[4][3], vel[4][3];
  load_tet(tv, b.rest, b.x, X);
#pragma unroll
  for (int a = 0; a < 4; a++) {
    const bool free = b.freeMask[vid[a]] != 0;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const size_t q = 3 * (size_t)vid[a] + i;
      vel[a][i] = free ? sp.nm[3] * (b.x[q] - b.xOld[q]) + sp.nm[4] * b.vOld[q] + sp.nm[5] * b.aOld[q] : 0.0;
    }
  }
  double F[9], Fd[9];
  deformation_gradient(X, Dinv, F);
  deformation_gradient(vel, Dinv, Fd);
  double G[9], P[9];  // G = F^T Fdot + Fdot^T F (symmetric), P = mu F G
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      double a = 0.0, c = 0.0;
#pragma unroll
      for (int k = 0; k < 3; k++) {
        a += F[k + 3 * i] * Fd[k + 3 * j];
        c += Fd[k + 3 * i] * F[k + 3 * j];
      }
      G[i + 3 * j] = a + c;
    }
#pragma unroll
  for (int j = 0; j < 3; j++)
#pragma unroll
    for (int i = 0; i < 3; i++)
      P[i + 3 * j] = sp.greenMu * (F[i] * G[3 * j] + F[i + 3] * G[1 + 3 * j] + F[i + 6] * G[2 + 3 * j]);
  double f[12];
  element_force(P, Dinv, b.vol[t], f);
  double* g = b.elemG + 12 * (size_t)t;
#pragma unroll
  for (int k = 0; k < 12; k++) g[k] += f[k];
}

// Standalone material terms of n elements (the VOLUME::HYPERELASTIC
// interface): psi, PK1, clampedHessian and the unclamped hessian, from F
// (svd_rv computed here) or, when Uin is given, from (U, Sigma, V) as the
// reference's overloads take them (HYPERELASTIC.h:37-49: F = U diag(Sigma)
// V^T for the F-form energies; ARAP and the eigensystems use the factors
// themselves).  Any output may be null.
__global__ void k_material_eval(MatParams m, int n, const double* Fin, const double* Uin, const double* Sin,
                                const double* Vin, double* psi, double* Pout, double* Hout, double* Huout) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= n) return;
  double F[9], U[9], S[3], V[9];
  if (Uin) {
#pragma unroll
    for (int k = 0; k < 9; k++) {
      U[k] = Uin[9 * (size_t)e + k];
      V[k] = Vin[9 * (size_t)e + k];
    }
#pragma unroll
    for (int k = 0; k < 3; k++) S[k] = Sin[3 * (size_t)e + k];
#pragma unroll
    for (int j = 0; j < 3; j++)
#pragma unroll
      for (int i = 0; i < 3; i++)
        F[i + 3 * j] = U[i] * S[0] * V[j] + U[i + 3] * S[1] * V[j + 3] + U[i + 6] * S[2] * V[j + 6];
  } else {
#pragma unroll
    for (int k = 0; k < 9; k++) F[k] = Fin[9 * (size_t)e + k];
    svd3_rv_fast(F, U, S, V);
  }
  if (is_anisotropic(m.kind)) {
    double g[3];
    const double I5 = aniso_stretch(m, F, g);
    const double I4 = aniso_invariant4(m, S, V);
    if (psi) psi[e] = aniso_psi(m, I5, I4);
    if (Pout) {
      const double sc = aniso_pk1_scale(m, I5, I4);
#pragma unroll
      for (int j = 0; j < 3; j++)
#pragma unroll
        for (int i = 0; i < 3; i++) Pout[9 * (size_t)e + i + 3 * j] = sc * (g[i] * m.a[j]);
    }
    if (Hout) aniso_hessian9(m, F, I4, true, Hout + 81 * (size_t)e);
    if (Huout) aniso_hessian9(m, F, I4, false, Huout + 81 * (size_t)e);
    return;
  }
  if (psi) psi[e] = material_psi(m, F, S);
  if (Pout) material_pk1(m, F, U, V, Pout + 9 * (size_t)e);
  const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  if (Hout) {
    double Hr[45];
    reduced_hessian<double>(m, U, S, V, I3, Hr);
    reduced_to_h9(Hr, Hout + 81 * (size_t)e);
  }
  if (Huout) {
    double Hr[45];
    reduced_hessian<double>(m, U, S, V, I3, Hr, false);
    reduced_to_h9(Hr, Huout + 81 * (size_t)e);
  }
}

// Standalone: per-tet F, sigma, element force and full 12x12 element Hessian.
__global__ void k_element_eval(int nt, const int4* tets, const double* rest, const double* x, const double* DmInv,
                               const double* volume, MatParams m, double* Fo, double* So, double* fo, double* Ho) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  double Dinv[9];
#pragma unroll
  for (int k = 0; k < 9; k++) Dinv[k] = DmInv[9 * (size_t)t + k];
  const double vol = volume[t];
  double X[4][3];
  load_tet(tets[t], rest, x, X);
  double F[9], U[9], S[3], V[9], P[9], f[12];
  deformation_gradient(X, Dinv, F);
  svd3_rv_fast(F, U, S, V);
  if (Fo)
    for (int k = 0; k < 9; k++) Fo[9 * (size_t)t + k] = F[k];
  if (So)
    for (int k = 0; k < 3; k++) So[3 * (size_t)t + k] = S[k];
  const bool aniso = is_anisotropic(m.kind);
  double g[3], c[4], I5 = 0.0, I4 = 0.0;
  if (aniso) {
    I5 = aniso_stretch(m, F, g);
    I4 = aniso_invariant4(m, S, V);
    for (int a = 0; a < 3; a++) c[a + 1] = Dinv[a] * m.a[0] + Dinv[a + 3] * m.a[1] + Dinv[a + 6] * m.a[2];
    c[0] = -(c[1] + c[2] + c[3]);
  }
  if (fo) {
    if (aniso) {
      const double sc = aniso_pk1_scale(m, I5, I4);
      for (int a = 0; a < 4; a++)
        for (int i = 0; i < 3; i++) f[3 * a + i] = -vol * sc * c[a] * g[i];
    } else {
      material_pk1(m, F, U, V, P);
      element_force(P, Dinv, vol, f);
    }
    for (int k = 0; k < 12; k++) fo[12 * (size_t)t + k] = f[k];
  }
  if (Ho) {
    double blk[kElemHess];
    if (aniso) {
      double al, be;
      const double a2 = m.a[0] * m.a[0] + m.a[1] * m.a[1] + m.a[2] * m.a[2];
      aniso_hessian_coeffs(m, I5, I4, I5 * a2, true, al, be);
      for (int A = 0; A < 4; A++)
        for (int B = A; B < 4; B++)
          for (int i = 0; i < 3; i++)
            for (int k = 0; k < 3; k++)
              blk[9 * upper_block(A, B) + 3 * i + k] = -vol * c[A] * c[B] * ((i == k ? al : 0.0) + be * g[i] * g[k]);
    } else {
      double Hr[45];
      reduced_hessian<double>(m, U, S, V, Dinv, Hr);
      expand_blocks<double, double>(Hr, vol, blk);
    }
    double* H = Ho + 144 * (size_t)t;
    for (int a = 0; a < 4; a++)
      for (int bb = 0; bb < 4; bb++)
        for (int i = 0; i < 3; i++)
          for (int k = 0; k < 3; k++) {
            const double val = (a <= bb) ? blk[9 * upper_block(a, bb) + 3 * i + k]
                                         : blk[9 * upper_block(bb, a) + 3 * k + i];
            H[(3 * a + i) + 12 * (3 * bb + k)] = val;
          }
  }
}

// Per-tet energy density times rest volume.
__global__ void k_energy(DeviceBatch b) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nt) return;
  const SceneParams& sp = b.scenes[b.tetScene[t]];
  const MatParams m = make_material(sp.kind, sp.mu, sp.lambda, sp.fiber);
  double Dinv[9];
  for (int k = 0; k < 9; k++) Dinv[k] = b.DmInv[9 * (size_t)t + k];
  double X[4][3];
  load_tet(b.tets[t], b.rest, b.x, X);
  double F[9], U[9], S[3], V[9];
  deformation_gradient(X, Dinv, F);
  svd3_rv_fast(F, U, S, V);
  double psi;
  if (is_anisotropic(m.kind)) {
    double g[3];
    const double I5 = aniso_stretch(m, F, g);
    psi = aniso_psi(m, I5, aniso_invariant4(m, S, V));
  } else {
    // isotropic energies keep the reparameterised constants of the scene
    const MatParams mi{sp.kind, sp.mu, sp.lambda, sp.alpha};
    psi = material_psi(mi, F, S);
  }
  b.psi[t] = b.vol[t] * psi;
}

}  // namespace

// CTA size: the batch's autotuned elemThreads (64 or 128; the kernels are
// bounded for 128).
// dynamic shared memory of a k_element CTA: 6 doubles per staged vertex
// (stageMax: the most distinct vertices of any pair of staging blocks)
static size_t stage_bytes(const DeviceBatch& b) { return sizeof(double) * 6 * (size_t)b.stageMax; }

void launch_element(const DeviceBatch& b, cudaStream_t s, int rawForces) {
  if (b.nt == 0) return;
  const int nt = b.elemThreads;
  k_element<double, kElemAll><<<(b.nt + nt - 1) / nt, nt, stage_bytes(b), s>>>(b, rawForces, b.elemH);
  if (b.anyAniso) k_element_aniso<double><<<(b.nt + 127) / 128, 128, 0, s>>>(b, rawForces, b.elemH);
}

void launch_element_mixed(const DeviceBatch& b, cudaStream_t s) {
  if (b.nt == 0) return;
  const int nt = b.elemThreads;
  if (b.anySvdFree)
    k_element<float, kElemSvdFree><<<(b.nt + nt - 1) / nt, nt, stage_bytes(b), s>>>(b, 0, b.elemHf);
  if (b.anyArap) k_element<float, kElemArap><<<(b.nt + nt - 1) / nt, nt, stage_bytes(b), s>>>(b, 0, b.elemHf);
  if (b.anyAniso) k_element_aniso<float><<<(b.nt + 127) / 128, 128, 0, s>>>(b, 0, b.elemHf);
}

void launch_green_damping(const DeviceBatch& b, cudaStream_t s) {
  if (b.nt == 0 || !b.anyGreen) return;
  k_green_damping<<<(b.nt + 127) / 128, 128, 0, s>>>(b);
}

void launch_energy(const DeviceBatch& b, cudaStream_t s) {
  if (b.nt == 0) return;
  k_energy<<<(b.nt + 127) / 128, 128, 0, s>>>(b);
}

void launch_material_eval(int kind, double mu, double lambda, const double* fiber, int n, const double* F,
                          const double* U, const double* S, const double* V, double* psi, double* P, double* H,
                          double* Hu, cudaStream_t s) {
  if (n <= 0) return;
  k_material_eval<<<(n + 127) / 128, 128, 0, s>>>(make_material(kind, mu, lambda, fiber), n, F, U, S, V, psi, P,
                                                   H, Hu);
}

void launch_element_eval(int nt, const int4* tets, const double* rest, const double* x, const double* DmInv,
                         const double* vol, int kind, double mu, double lambda, const double* fiber, double* F,
                         double* sigma, double* force, double* hessian, cudaStream_t s) {
  if (nt <= 0) return;
  k_element_eval<<<(nt + 127) / 128, 128, 0, s>>>(nt, tets, rest, x, DmInv, vol,
                                                   make_material(kind, mu, lambda, fiber), F, sigma, force, hessian);
}

}  // namespace hobak
