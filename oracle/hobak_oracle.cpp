// CPU restatement of HOBAK's implicit tet-FEM timestep (the oracle).
//
// TEST INFRASTRUCTURE.  Only tests/, __graft_entry__.smoke() and bench.py's
// CPU-baseline leg load this library, and only as the checker or the timed CPU
// baseline -- never as the product path.  It is an independent FP64
// restatement of the reference algorithm (no Eigen, no shared code with the
// CUDA library), pinned against the reference build's golden vectors in
// tests/golden/.  Each function cites the reference file:line it follows.
//
// Layouts: vectors are interleaved xyz (3V doubles); 3x3 matrices are column
// major (a[i + 3*j] = A(i,j)), like the reference's flatten()
// (util/MATRIX_UTIL.cpp:33-43); 9x9 and 12x12 matrices are column major.
// Sparse matrices are 3x3-block CSR (BSR) with blocks stored column major.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <array>
#include <limits>
#include <map>
#include <numeric>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

enum Material {
  SNH = 0, ARAP = 1, STVK = 2, LINEAR = 3, NHBW = 4, SNHB = 5,
  // anisotropic energies along a fibre direction a (Hyperelastic/Volume/ANISOTROPIC_*.cpp)
  AARAP = 6, ASTVK = 7, AFUNG = 8, ADIR = 9
};
inline bool anisotropic(int kind) { return kind >= AARAP && kind <= ADIR; }

inline double det3(const double* A) {
  return A[0] * (A[4] * A[8] - A[7] * A[5]) - A[3] * (A[1] * A[8] - A[7] * A[2]) +
         A[6] * (A[1] * A[5] - A[4] * A[2]);
}

// C = A * B (3x3, column major)
inline void mul3(const double* A, const double* B, double* C) {
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += A[i + 3 * k] * B[k + 3 * j];
      C[i + 3 * j] = s;
    }
}

// C = A * B^T
inline void mul3t(const double* A, const double* B, double* C) {
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += A[i + 3 * k] * B[j + 3 * k];
      C[i + 3 * j] = s;
    }
}

// 3x3 inverse by cofactors (TET_MESH.cpp:178-191 uses Eigen's Dm.inverse())
inline void inv3(const double* A, double* Ai) {
  const double d = det3(A);
  const double id = 1.0 / d;
  Ai[0] = (A[4] * A[8] - A[5] * A[7]) * id;
  Ai[1] = (A[2] * A[7] - A[1] * A[8]) * id;
  Ai[2] = (A[1] * A[5] - A[2] * A[4]) * id;
  Ai[3] = (A[5] * A[6] - A[3] * A[8]) * id;
  Ai[4] = (A[0] * A[8] - A[2] * A[6]) * id;
  Ai[5] = (A[2] * A[3] - A[0] * A[5]) * id;
  Ai[6] = (A[3] * A[7] - A[4] * A[6]) * id;
  Ai[7] = (A[1] * A[6] - A[0] * A[7]) * id;
  Ai[8] = (A[0] * A[4] - A[1] * A[3]) * id;
}

// Rotation-variant SVD, F = U diag(S) V^T with S sorted by magnitude, U and V
// rotations, and any reflection carried by the sign of S[2] -- the convention
// of svd_rv (util/MATRIX_UTIL.cpp:76-95).  Computed by one-sided (Hestenes)
// Jacobi orthogonalisation of F's columns, a different route from the
// reference's two-sided JacobiSVD; the factors agree up to the usual
// non-uniqueness, and everything downstream is invariant to that.
void svd_rv(const double* F, double* U, double* S, double* V) {
  double A[9];
  std::memcpy(A, F, sizeof(A));
  double W[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
  const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 40; sweep++) {
    bool rotated = false;
    for (int r = 0; r < 3; r++) {
      const int p = pq[r][0], q = pq[r][1];
      double* ap = A + 3 * p;
      double* aq = A + 3 * q;
      const double alpha = ap[0] * ap[0] + ap[1] * ap[1] + ap[2] * ap[2];
      const double beta = aq[0] * aq[0] + aq[1] * aq[1] + aq[2] * aq[2];
      const double gamma = ap[0] * aq[0] + ap[1] * aq[1] + ap[2] * aq[2];
      if (gamma == 0.0 || std::fabs(gamma) <= 1e-15 * std::sqrt(alpha * beta)) continue;
      rotated = true;
      const double zeta = (beta - alpha) / (2.0 * gamma);
      const double t = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
      const double c = 1.0 / std::sqrt(1.0 + t * t), s = c * t;
      for (int i = 0; i < 3; i++) {
        const double x = ap[i], y = aq[i];
        ap[i] = c * x - s * y;
        aq[i] = s * x + c * y;
        const double vx = W[i + 3 * p], vy = W[i + 3 * q];
        W[i + 3 * p] = c * vx - s * vy;
        W[i + 3 * q] = s * vx + c * vy;
      }
    }
    if (!rotated) break;
  }
  double sig[3];
  for (int k = 0; k < 3; k++)
    sig[k] = std::sqrt(A[3 * k] * A[3 * k] + A[3 * k + 1] * A[3 * k + 1] + A[3 * k + 2] * A[3 * k + 2]);
  int order[3] = {0, 1, 2};
  std::sort(order, order + 3, [&](int a, int b) { return sig[a] > sig[b]; });
  for (int k = 0; k < 3; k++) {
    const int o = order[k];
    S[k] = sig[o];
    for (int i = 0; i < 3; i++) {
      V[i + 3 * k] = W[i + 3 * o];
      U[i + 3 * k] = S[k] > 0 ? A[i + 3 * o] / S[k] : 0.0;
    }
  }
  // complete U where columns vanished (rank-deficient F)
  const double tiny = 1e-300;
  if (S[0] <= tiny) {
    const double I[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    std::memcpy(U, I, sizeof(I));
  } else if (S[1] <= tiny) {
    // any unit vector orthogonal to u0
    const double* u0 = U;
    double e[3] = {0, 0, 0};
    int m = 0;
    for (int i = 1; i < 3; i++)
      if (std::fabs(u0[i]) < std::fabs(u0[m])) m = i;
    e[m] = 1;
    double d = e[0] * u0[0] + e[1] * u0[1] + e[2] * u0[2];
    double u1[3] = {e[0] - d * u0[0], e[1] - d * u0[1], e[2] - d * u0[2]};
    double n = std::sqrt(u1[0] * u1[0] + u1[1] * u1[1] + u1[2] * u1[2]);
    for (int i = 0; i < 3; i++) U[3 + i] = u1[i] / n;
  }
  if (S[2] <= tiny || S[1] <= tiny || S[0] <= tiny) {
    U[6] = U[1] * U[5] - U[2] * U[4];
    U[7] = U[2] * U[3] - U[0] * U[5];
    U[8] = U[0] * U[4] - U[1] * U[3];
  }
  // fold reflections into S[2]
  if (det3(U) < 0) {
    for (int i = 0; i < 3; i++) U[6 + i] = -U[6 + i];
    S[2] = -S[2];
  }
  if (det3(V) < 0) {
    for (int i = 0; i < 3; i++) V[6 + i] = -V[6 + i];
    S[2] = -S[2];
  }
}

// Symmetric 3x3 eigensystem by cyclic Jacobi rotations; A = Q diag(L) Q^T.
// Stands in for Eigen::SelfAdjointEigenSolver<MATRIX3> (SNH.cpp:130).
void eig3sym(const double* Ain, double* Q, double* L) {
  double a[3][3];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) a[i][j] = Ain[i + 3 * j];
  double q[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
  const int pq[3][2] = {{0, 1}, {0, 2}, {1, 2}};
  for (int sweep = 0; sweep < 50; sweep++) {
    double off = std::fabs(a[0][1]) + std::fabs(a[0][2]) + std::fabs(a[1][2]);
    double diag = std::fabs(a[0][0]) + std::fabs(a[1][1]) + std::fabs(a[2][2]);
    if (off == 0.0 || off <= 1e-15 * diag) break;
    for (int r = 0; r < 3; r++) {
      const int p = pq[r][0], k = pq[r][1];
      if (a[p][k] == 0.0) continue;
      const double theta = (a[k][k] - a[p][p]) / (2.0 * a[p][k]);
      const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
      const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
      // a <- J^T a J, J = rotation in the (p,k) plane
      for (int m = 0; m < 3; m++) {
        const double amp = a[m][p], amk = a[m][k];
        a[m][p] = c * amp - s * amk;
        a[m][k] = s * amp + c * amk;
      }
      for (int m = 0; m < 3; m++) {
        const double apm = a[p][m], akm = a[k][m];
        a[p][m] = c * apm - s * akm;
        a[k][m] = s * apm + c * akm;
      }
      for (int m = 0; m < 3; m++) {
        const double qmp = q[m][p], qmk = q[m][k];
        q[m][p] = c * qmp - s * qmk;
        q[m][k] = s * qmp + c * qmk;
      }
    }
  }
  for (int i = 0; i < 3; i++) {
    L[i] = a[i][i];
    for (int m = 0; m < 3; m++) Q[m + 3 * i] = q[m][i];
  }
}

struct MaterialParams {
  int kind;
  double mu, lambda, alpha;
  double a[3];  // anisotropic energies: unit fibre direction (the constructor normalises it)
};

MaterialParams makeMaterial(int kind, double mu, double lambda, const double* fiber = nullptr) {
  MaterialParams m{kind, mu, lambda, 0.0, {1.0, 0.0, 0.0}};
  if (fiber) {  // ANISOTROPIC_ARAP.cpp:26-29 (_a.normalize(), _A = a a^T)
    const double n = std::sqrt(fiber[0] * fiber[0] + fiber[1] * fiber[1] + fiber[2] * fiber[2]);
    for (int i = 0; i < 3; i++) m.a[i] = n > 0.0 ? fiber[i] / n : fiber[i];
  }
  if (kind == SNH) {  // SNH.cpp:23-32
    m.lambda = lambda + mu;
    m.alpha = 1.0 + m.mu / m.lambda;
  } else if (kind == NHBW) {  // NEO_HOOKEAN_BW.cpp:23-29
    m.alpha = 1.0 + mu / lambda;
  } else if (kind == SNHB) {  // SNH_WITH_BARRIER.cpp:26-35
    m.mu = (4.0 / 3.0) * mu;
    m.lambda = lambda + (5.0 / 6.0) * mu;
    m.alpha = 1.0 + m.mu / m.lambda - m.mu / (4.0 * m.lambda);
  }
  return m;
}

// pJ/pF = [f1 x f2, f2 x f0, f0 x f1] (util/MATRIX_UTIL.cpp:561-568)
inline void pJpF(const double* F, double* G) {
  const double* f0 = F;
  const double* f1 = F + 3;
  const double* f2 = F + 6;
  G[0] = f1[1] * f2[2] - f1[2] * f2[1];
  G[1] = f1[2] * f2[0] - f1[0] * f2[2];
  G[2] = f1[0] * f2[1] - f1[1] * f2[0];
  G[3] = f2[1] * f0[2] - f2[2] * f0[1];
  G[4] = f2[2] * f0[0] - f2[0] * f0[2];
  G[5] = f2[0] * f0[1] - f2[1] * f0[0];
  G[6] = f0[1] * f1[2] - f0[2] * f1[1];
  G[7] = f0[2] * f1[0] - f0[0] * f1[2];
  G[8] = f0[0] * f1[1] - f0[1] * f1[0];
}

inline double sqnorm9(const double* A) {
  double s = 0;
  for (int k = 0; k < 9; k++) s += A[k] * A[k];
  return s;
}

// Anisotropic energies (ANISOTROPIC_ARAP/STVK/FUNG/DIRICHLET.cpp): with the
// unit fibre direction a, g = F a, F A = g a^T (A = a a^T) and
// I5 = |F a|^2 (invariant5, MATRIX_UTIL.cpp:553-556).  Every stress is a
// scalar times F A, every Hessian alpha H5 + beta fa fa^T with
// H5 = kronIdentity(A) (MATRIX_UTIL.cpp:512-524) and fa = vec(F A).
void fiberTerms(const MaterialParams& m, const double* F, double* g, double* FA, double& I5) {
  for (int i = 0; i < 3; i++) g[i] = F[i] * m.a[0] + F[i + 3] * m.a[1] + F[i + 6] * m.a[2];
  I5 = g[0] * g[0] + g[1] * g[1] + g[2] * g[2];
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) {
      double s = 0;
      for (int k = 0; k < 3; k++) s += F[i + 3 * k] * (m.a[k] * m.a[j]);
      FA[i + 3 * j] = s;
    }
}

// I4 = a^T (V Sigma V^T) a with svd_rv (invariant4, MATRIX_UTIL.cpp:545-552);
// only its sign and magnitude near 0 are used
double invariant4(const MaterialParams& m, const double* F) {
  double U[9], S[3], V[9];
  svd_rv(F, U, S, V);
  double I4 = 0;
  for (int k = 0; k < 3; k++) {
    const double va = V[3 * k] * m.a[0] + V[3 * k + 1] * m.a[1] + V[3 * k + 2] * m.a[2];
    I4 += S[k] * va * va;
  }
  return I4;
}

double psiAniso(const MaterialParams& m, const double* F) {
  double g[3], FA[9], I5;
  fiberTerms(m, F, g, FA, I5);
  switch (m.kind) {
    case AARAP: {  // ANISOTROPIC_ARAP.cpp:40-47
      const double SI4 = invariant4(m, F) > 0.0 ? 1.0 : -1.0;
      const double diff = std::sqrt(I5) - SI4;
      return 0.5 * m.mu * diff * diff;
    }
    case ASTVK: return 0.5 * m.mu * (I5 - 1.0) * (I5 - 1.0);   // ANISOTROPIC_STVK.cpp:42-46
    case AFUNG: return m.mu * (std::exp(I5 - 1.0) - I5);       // ANISOTROPIC_FUNG.cpp:40-44
    default: return m.mu * I5;                                 // ANISOTROPIC_DIRICHLET.cpp:36-39
  }
}

// P = s(F) F A: ANISOTROPIC_ARAP.cpp:52-65 (with its |I4| < 1e-8 branch),
// ANISOTROPIC_STVK.cpp:51-55, ANISOTROPIC_FUNG.cpp:50-54, ANISOTROPIC_DIRICHLET.cpp:44-47
void PK1Aniso(const MaterialParams& m, const double* F, double* P) {
  double g[3], FA[9], I5, sc;
  fiberTerms(m, F, g, FA, I5);
  switch (m.kind) {
    case AARAP: {
      const double I4 = invariant4(m, F);
      const double SI4 = I4 > 0.0 ? 1.0 : -1.0;
      sc = std::fabs(I4) >= 1e-8 ? m.mu * (1.0 - SI4 / std::sqrt(I5)) : -1.0 * m.mu * (1.0 - 1.0 / 2.0);
      break;
    }
    case ASTVK: sc = 2.0 * m.mu * (I5 - 1.0); break;
    case AFUNG: sc = 2.0 * m.mu * (std::exp(I5 - 1.0) - 1.0); break;
    default: sc = 2.0 * m.mu; break;
  }
  for (int k = 0; k < 9; k++) P[k] = sc * FA[k];
}

// (alpha, beta) of the Hessian alpha H5 + beta fa fa^T, clamped or not:
// ANISOTROPIC_ARAP.cpp:70-110, ANISOTROPIC_STVK.cpp:60-100,
// ANISOTROPIC_FUNG.cpp:60-105, ANISOTROPIC_DIRICHLET.cpp:52-77.
void hessianAnisoCoeffs(const MaterialParams& m, const double* F, bool clamp, double& al, double& be) {
  double g[3], FA[9], I5;
  fiberTerms(m, F, g, FA, I5);
  const double fa2 = sqnorm9(FA);
  switch (m.kind) {
    case AARAP: {
      const double SI4 = invariant4(m, F) > 0.0 ? 1.0 : -1.0;
      if (!clamp || I5 >= SI4) {
        const double si = 1.0 / std::sqrt(I5);
        al = m.mu * (1.0 - SI4 * si);
        be = m.mu * (SI4 * si * si * si);
      } else {
        al = 0.0;
        be = m.mu * (1.0 / I5);
      }
      return;
    }
    case ASTVK:
    case AFUNG: {
      const double e = m.kind == AFUNG ? std::exp(I5 - 1.0) : 1.0;
      const double l1 = m.kind == AFUNG ? 2.0 * m.mu * (e - 1.0) : 2.0 * m.mu * (I5 - 1.0);
      const double l0 = m.kind == AFUNG ? l1 + 4.0 * m.mu * I5 * e : l1 + 4.0 * m.mu * I5;
      if (!clamp || (l0 > 0.0 && l1 > 0.0)) {
        al = l1;
        be = 4.0 * m.mu * e;
      } else if (l0 < 0.0) {
        al = be = 0.0;
      } else {  // lambda0 along fa / |fa| (Eigen's normalized(): fa itself when |fa| = 0)
        al = 0.0;
        be = fa2 > 0.0 ? l0 / fa2 : l0;
      }
      return;
    }
    default:
      al = 2.0 * m.mu;
      be = 0.0;
      return;
  }
}

void hessianAniso(const MaterialParams& m, const double* F, bool clamp, double* H9) {
  double g[3], FA[9], I5, al, be;
  fiberTerms(m, F, g, FA, I5);
  hessianAnisoCoeffs(m, F, clamp, al, be);
  for (int c = 0; c < 9; c++)
    for (int r = 0; r < 9; r++) {
      const double h5 = (r % 3 == c % 3) ? m.a[r / 3] * m.a[c / 3] : 0.0;
      H9[r + 9 * c] = al * h5 + be * FA[r] * FA[c];
    }
}

// Strain energy density psi(F): SNH.cpp:34-43, ARAP.cpp:39-43 (through
// HYPERELASTIC.cpp:41-47), STVK.cpp psi, LINEAR.cpp psi, NEO_HOOKEAN_BW.cpp psi,
// SNH_WITH_BARRIER.cpp psi.
double psi(const MaterialParams& m, const double* F) {
  if (anisotropic(m.kind)) return psiAniso(m, F);
  switch (m.kind) {
    case SNH: {
      const double Ic = sqnorm9(F), Jm = det3(F) - m.alpha;
      return 0.5 * (m.mu * (Ic - 3.0) + m.lambda * Jm * Jm);
    }
    case ARAP: {
      double U[9], S[3], V[9], R[9];
      svd_rv(F, U, S, V);
      mul3t(U, V, R);
      double d = 0;
      for (int k = 0; k < 9; k++) d += (F[k] - R[k]) * (F[k] - R[k]);
      return m.mu * d;
    }
    case STVK: {
      double FtF[9], E[9];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          double s = 0;
          for (int k = 0; k < 3; k++) s += F[k + 3 * i] * F[k + 3 * j];
          FtF[i + 3 * j] = s;
        }
      for (int k = 0; k < 9; k++) E[k] = 0.5 * (FtF[k] - (k % 4 == 0 ? 1.0 : 0.0));
      const double tr = E[0] + E[4] + E[8];
      return m.mu * sqnorm9(E) + m.lambda * 0.5 * tr * tr;
    }
    case LINEAR: {
      double e[9];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) e[i + 3 * j] = 0.5 * (F[i + 3 * j] + F[j + 3 * i]) - (i == j ? 1.0 : 0.0);
      const double tr = e[0] + e[4] + e[8];
      return m.mu * sqnorm9(e) + 0.5 * m.lambda * tr * tr;
    }
    case NHBW: {
      const double Ic = sqnorm9(F), lj = std::log(det3(F));
      return m.mu * 0.5 * (Ic - 3.0) - m.mu * lj + m.lambda * 0.5 * lj * lj;
    }
    case SNHB: {
      const double Ic = sqnorm9(F), Jm = det3(F) - m.alpha;
      return 0.5 * (m.mu * (Ic - 3.0) + m.lambda * Jm * Jm - m.mu * std::log(Ic + 1.0));
    }
  }
  return 0.0;
}

// First Piola-Kirchhoff stress P(F): SNH.cpp:45-50, ARAP.cpp:48-55 (through
// HYPERELASTIC.cpp:61-67), STVK.cpp PK1, LINEAR.cpp PK1, NEO_HOOKEAN_BW.cpp PK1,
// SNH_WITH_BARRIER.cpp PK1.
void PK1(const MaterialParams& m, const double* F, double* P) {
  if (anisotropic(m.kind)) return PK1Aniso(m, F, P);
  switch (m.kind) {
    case SNH: {
      double G[9];
      pJpF(F, G);
      const double Jm = det3(F) - m.alpha;
      for (int k = 0; k < 9; k++) P[k] = m.mu * F[k] + m.lambda * Jm * G[k];
      return;
    }
    case ARAP: {
      // R (2 mu (S - I)) with R = U V^T, S = V Sigma V^T
      double U[9], S[3], V[9], R[9], Sm[9], T[9];
      svd_rv(F, U, S, V);
      mul3t(U, V, R);
      double VS[9];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) VS[i + 3 * j] = V[i + 3 * j] * S[j];
      mul3t(VS, V, Sm);
      for (int k = 0; k < 9; k++) T[k] = 2.0 * m.mu * (Sm[k] - (k % 4 == 0 ? 1.0 : 0.0));
      mul3(R, T, P);
      return;
    }
    case STVK: {
      double FtF[9], E[9], Sg[9];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
          double s = 0;
          for (int k = 0; k < 3; k++) s += F[k + 3 * i] * F[k + 3 * j];
          FtF[i + 3 * j] = s;
        }
      for (int k = 0; k < 9; k++) E[k] = 0.5 * (FtF[k] - (k % 4 == 0 ? 1.0 : 0.0));
      const double tr = E[0] + E[4] + E[8];
      for (int k = 0; k < 9; k++) Sg[k] = (k % 4 == 0 ? m.lambda * tr : 0.0) + 2.0 * m.mu * E[k];
      mul3(F, Sg, P);
      return;
    }
    case LINEAR: {
      double e[9];
      for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) e[i + 3 * j] = 0.5 * (F[i + 3 * j] + F[j + 3 * i]) - (i == j ? 1.0 : 0.0);
      const double tr = e[0] + e[4] + e[8];
      for (int k = 0; k < 9; k++) P[k] = 2.0 * m.mu * e[k] + (k % 4 == 0 ? m.lambda * tr : 0.0);
      return;
    }
    case NHBW: {
      double G[9];
      pJpF(F, G);
      const double J = det3(F);
      for (int k = 0; k < 9; k++) P[k] = m.mu * (F[k] - (1.0 / J) * G[k]) + m.lambda * std::log(J) * (1.0 / J) * G[k];
      return;
    }
    case SNHB: {
      double G[9];
      pJpF(F, G);
      const double Ic = sqnorm9(F), Jm = det3(F) - m.alpha;
      for (int k = 0; k < 9; k++) P[k] = m.mu * F[k] + m.lambda * Jm * G[k] - m.mu / (Ic + 1) * F[k];
      return;
    }
  }
}

// Q9 columns 0-5: twist and flip modes (util/MATRIX_UTIL.cpp:420-460)
void twistFlip(const double* U, const double* V, double* Q9) {
  const double r = 1.0 / std::sqrt(2.0);
  // twist k is U T_k V^T with T_k = e_j e_i^T - e_i e_j^T for (i, j) =
  // (1,2), (2,0), (1,0): the x-, y- and z-twists of MATRIX_UTIL.cpp:424-433
  const int ij[3][2] = {{1, 2}, {2, 0}, {1, 0}};
  for (int k = 0; k < 3; k++) {
    const int i = ij[k][0], j = ij[k][1];
    for (int c = 0; c < 3; c++)
      for (int rr = 0; rr < 3; rr++) {
        // (U T V^T)(rr,c) = U(rr,j) V(c,i) - U(rr,i) V(c,j)
        const double tw = U[rr + 3 * j] * V[c + 3 * i] - U[rr + 3 * i] * V[c + 3 * j];
        const double fl = U[rr + 3 * j] * V[c + 3 * i] + U[rr + 3 * i] * V[c + 3 * j];
        Q9[9 * k + rr + 3 * c] = r * tw;
        Q9[9 * (k + 3) + rr + 3 * c] = r * fl;
      }
  }
}

// Q9 columns 6-8: scaling modes U diag(q_k) V^T (util/MATRIX_UTIL.cpp:465-497)
void scaling(const double* U, const double* Q3, const double* V, double* Q9) {
  for (int k = 0; k < 3; k++)
    for (int c = 0; c < 3; c++)
      for (int rr = 0; rr < 3; rr++) {
        double s = 0;
        for (int m = 0; m < 3; m++) s += U[rr + 3 * m] * Q3[m + 3 * k] * V[c + 3 * m];
        Q9[9 * (6 + k) + rr + 3 * c] = s;
      }
}

// H9 = Q diag(max(L, 0)) Q^T (clamp) or Q diag(L) Q^T
void assembleClamped(const double* Q9, double* L, double* H9, bool clamp = true) {
  for (int k = 0; k < 9; k++)
    if (clamp && L[k] < 0.0) L[k] = 0.0;
  for (int c = 0; c < 9; c++)
    for (int r = 0; r < 9; r++) {
      double s = 0;
      for (int k = 0; k < 9; k++) s += Q9[9 * k + r] * L[k] * Q9[9 * k + c];
      H9[r + 9 * c] = s;
    }
}

// Clamped 9x9 Hessian d2psi/dF2 projected to PSD, as a function of
// (U, Sigma, V): SNH.cpp:94-144, ARAP.cpp:113-135, STVK.cpp buildEigensystem
// (Appendix F.1 eigensystem), LINEAR.cpp hessian (no clamp),
// NEO_HOOKEAN_BW.cpp clampedHessian, SNH_WITH_BARRIER.cpp clampedHessian.
// With clamp = false the same eigensystem gives the unclamped Hessian
// (SNH.cpp, STVK.cpp, LINEAR.cpp, NEO_HOOKEAN_BW.cpp, SNH_WITH_BARRIER.cpp
// hessian(F); ARAP.cpp hessian(U, Sigma, V)).  Anisotropic energies take the
// F-form through F = U diag(Sigma) V^T, as HYPERELASTIC.cpp:99-103 does.
void eigenHessian(const MaterialParams& m, const double* U, const double* S, const double* V, double* H9,
                  bool clamp) {
  if (anisotropic(m.kind)) {
    double US[9], F[9];
    for (int j = 0; j < 3; j++)
      for (int i = 0; i < 3; i++) US[i + 3 * j] = U[i + 3 * j] * S[j];
    mul3t(US, V, F);
    hessianAniso(m, F, clamp, H9);
    return;
  }
  double Q9[81], L[9];
  const double s0 = S[0], s1 = S[1], s2 = S[2];
  if (m.kind == LINEAR) {
    std::memset(H9, 0, 81 * sizeof(double));
    for (int k = 0; k < 9; k++) H9[k + 9 * k] = m.mu;
    const double d = m.mu + m.lambda;
    H9[0 + 9 * 0] += d;
    H9[4 + 9 * 4] += d;
    H9[8 + 9 * 8] += d;
    H9[1 + 9 * 3] = H9[3 + 9 * 1] = m.mu;
    H9[2 + 9 * 6] = H9[6 + 9 * 2] = m.mu;
    H9[5 + 9 * 7] = H9[7 + 9 * 5] = m.mu;
    H9[0 + 9 * 4] = H9[0 + 9 * 8] = H9[4 + 9 * 8] = m.lambda;
    H9[4 + 9 * 0] = H9[8 + 9 * 0] = H9[8 + 9 * 4] = m.lambda;
    return;
  }
  twistFlip(U, V, Q9);
  if (m.kind == ARAP) {
    for (int k = 0; k < 9; k++) L[k] = 2.0 * m.mu;
    L[0] = m.mu * (2.0 - 4.0 / (s1 + s2));
    L[1] = m.mu * (2.0 - 4.0 / (s0 + s2));
    L[2] = m.mu * (2.0 - 4.0 / (s0 + s1));
    const double I3[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    scaling(U, I3, V, Q9);
    assembleClamped(Q9, L, H9, clamp);
    return;
  }
  double A[9];
  if (m.kind == SNH) {
    const double J = s0 * s1 * s2;
    const double front = m.lambda * (J - 1.0) - m.mu;
    L[0] = front * s0 + m.mu;
    L[1] = front * s1 + m.mu;
    L[2] = front * s2 + m.mu;
    L[3] = -front * s0 + m.mu;
    L[4] = -front * s1 + m.mu;
    L[5] = -front * s2 + m.mu;
    A[0] = m.mu + m.lambda * s1 * s1 * s2 * s2;
    A[4] = m.mu + m.lambda * s0 * s0 * s2 * s2;
    A[8] = m.mu + m.lambda * s0 * s0 * s1 * s1;
    const double od = m.lambda * (2.0 * J - 1.0) - m.mu;
    A[3] = A[1] = od * s2;
    A[6] = A[2] = od * s1;
    A[7] = A[5] = od * s0;
  } else if (m.kind == STVK) {
    const double I2 = s0 * s0 + s1 * s1 + s2 * s2;
    const double front = -m.mu + m.lambda * 0.5 * (I2 - 3.0);
    L[0] = front + m.mu * (s1 * s1 + s2 * s2 - s1 * s2);
    L[1] = front + m.mu * (s0 * s0 + s2 * s2 - s0 * s2);
    L[2] = front + m.mu * (s0 * s0 + s1 * s1 - s0 * s1);
    L[3] = front + m.mu * (s1 * s1 + s2 * s2 + s1 * s2);
    L[4] = front + m.mu * (s0 * s0 + s2 * s2 + s0 * s2);
    L[5] = front + m.mu * (s0 * s0 + s1 * s1 + s0 * s1);
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++)
        A[i + 3 * j] = (i == j) ? front + (m.lambda + 3.0 * m.mu) * S[i] * S[i] : m.lambda * S[i] * S[j];
  } else if (m.kind == NHBW) {
    const double J = s0 * s1 * s2, lj = std::log(J);
    const double i01 = 1.0 / (s0 * s1), i02 = 1.0 / (s0 * s2), i12 = 1.0 / (s1 * s2);
    const double front = m.lambda * lj - m.mu;
    L[0] = front * i12 + m.mu;
    L[1] = front * i02 + m.mu;
    L[2] = front * i01 + m.mu;
    L[3] = -front * i12 + m.mu;
    L[4] = -front * i02 + m.mu;
    L[5] = -front * i01 + m.mu;
    const double fd = m.lambda * (1.0 - lj) + m.mu;
    A[0] = fd / (s0 * s0) + m.mu;
    A[4] = fd / (s1 * s1) + m.mu;
    A[8] = fd / (s2 * s2) + m.mu;
    A[3] = A[1] = m.lambda * i01;
    A[6] = A[2] = m.lambda * i02;
    A[7] = A[5] = m.lambda * i12;
  } else {  // SNHB
    const double J = s0 * s1 * s2, I2 = s0 * s0 + s1 * s1 + s2 * s2;
    const double front = -m.mu / (I2 + 1.0) + m.mu;
    const double back = m.lambda * (J - m.alpha);
    for (int i = 0; i < 3; i++) {
      L[i] = front + back * S[i];
      L[i + 3] = front - back * S[i];
    }
    const double sq = (I2 + 1.0) * (I2 + 1.0), isq = 1.0 / sq, tm = 2.0 * m.mu;
    const double fd = (-m.mu * (I2 + 1.0)) * isq + m.mu;
    const double fo = (2.0 * J - m.alpha) * m.lambda;
    A[0] = fd + tm * s0 * s0 * isq + m.lambda * s1 * s1 * s2 * s2;
    A[4] = fd + tm * s1 * s1 * isq + m.lambda * s0 * s0 * s2 * s2;
    A[8] = fd + tm * s2 * s2 * isq + m.lambda * s0 * s0 * s1 * s1;
    A[3] = A[1] = fo * s2 + (tm * s0 * s1) * isq;
    A[6] = A[2] = fo * s1 + (tm * s0 * s2) * isq;
    A[7] = A[5] = fo * s0 + (tm * s1 * s2) * isq;
  }
  double Q3[9], L3[3];
  eig3sym(A, Q3, L3);
  for (int k = 0; k < 3; k++) L[6 + k] = L3[k];
  scaling(U, Q3, V, Q9);
  assembleClamped(Q9, L, H9, clamp);
}

void clampedHessian(const MaterialParams& m, const double* U, const double* S, const double* V, double* H9) {
  eigenHessian(m, U, S, V, H9, true);
}

// pFpx (9x12) from DmInv (TET_MESH.cpp:197-252): column 3*a+i, row i+3*j.
void pFpx(const double* Dinv, double* P) {
  std::memset(P, 0, 108 * sizeof(double));
  for (int j = 0; j < 3; j++) {
    const double t = -(Dinv[0 + 3 * j] + Dinv[1 + 3 * j] + Dinv[2 + 3 * j]);
    for (int i = 0; i < 3; i++) {
      const int row = i + 3 * j;
      P[row + 9 * (0 + i)] = t;
      for (int a = 1; a < 4; a++) P[row + 9 * (3 * a + i)] = Dinv[(a - 1) + 3 * j];
    }
  }
}

struct Mesh {
  int nv = 0, nt = 0;
  std::vector<double> rest;     // 3V
  std::vector<int> tets;        // 4T
  std::vector<double> vol;      // T
  std::vector<double> oneRing;  // V
  std::vector<double> DmInv;    // 9T
  // BSR pattern: row u -> sorted neighbour vertices
  std::vector<int> rowptr, cols;
  std::vector<int> diag;        // block index of (u,u)
  // vertex -> incident (tet, local slot), ascending tet
  std::vector<int> vtxptr, vtxinc;
  // per tet: block index of (tet[a], tet[b]) for a,b in 0..3
  std::vector<int> tetBlocks;   // 16T
};

// Rest volumes, one-ring volumes, DmInv (TET_MESH.cpp:121-191) and the
// block sparsity of the stiffness matrix (TET_MESH_FASTER.cpp:30-73).
void buildMesh(Mesh& M, int nv, int nt, const double* rest, const int* tets) {
  M.nv = nv;
  M.nt = nt;
  M.rest.assign(rest, rest + 3 * nv);
  M.tets.assign(tets, tets + 4 * nt);
  M.vol.resize(nt);
  M.oneRing.assign(nv, 0.0);
  M.DmInv.resize(9 * (size_t)nt);
  for (int t = 0; t < nt; t++) {
    const int* v = tets + 4 * t;
    double Dm[9];
    for (int a = 0; a < 3; a++)
      for (int i = 0; i < 3; i++) Dm[i + 3 * a] = rest[3 * v[a + 1] + i] - rest[3 * v[0] + i];
    const double* d1 = Dm;
    const double* d2 = Dm + 3;
    const double* d3 = Dm + 6;
    const double cr[3] = {d1[1] * d2[2] - d1[2] * d2[1], d1[2] * d2[0] - d1[0] * d2[2], d1[0] * d2[1] - d1[1] * d2[0]};
    M.vol[t] = (d3[0] * cr[0] + d3[1] * cr[1] + d3[2] * cr[2]) / 6.0;
    inv3(Dm, &M.DmInv[9 * (size_t)t]);
  }
  for (int t = 0; t < nt; t++) {
    const double q = 0.25 * M.vol[t];
    for (int a = 0; a < 4; a++) M.oneRing[tets[4 * t + a]] += q;
  }
  // vertex incidence, ascending tet order
  M.vtxptr.assign(nv + 1, 0);
  for (int k = 0; k < 4 * nt; k++) M.vtxptr[tets[k] + 1]++;
  for (int v = 0; v < nv; v++) M.vtxptr[v + 1] += M.vtxptr[v];
  M.vtxinc.resize(4 * (size_t)nt);
  std::vector<int> fill(M.vtxptr.begin(), M.vtxptr.end() - 1);
  for (int t = 0; t < nt; t++)
    for (int a = 0; a < 4; a++) M.vtxinc[fill[tets[4 * t + a]]++] = 4 * t + a;
  // block pattern
  M.rowptr.assign(nv + 1, 0);
  std::vector<std::vector<int>> nb(nv);
  for (int v = 0; v < nv; v++) {
    auto& n = nb[v];
    for (int k = M.vtxptr[v]; k < M.vtxptr[v + 1]; k++) {
      const int t = M.vtxinc[k] / 4;
      for (int b = 0; b < 4; b++) n.push_back(tets[4 * t + b]);
    }
    std::sort(n.begin(), n.end());
    n.erase(std::unique(n.begin(), n.end()), n.end());
    M.rowptr[v + 1] = M.rowptr[v] + (int)n.size();
  }
  M.cols.resize(M.rowptr[nv]);
  M.diag.resize(nv);
  for (int v = 0; v < nv; v++) {
    std::copy(nb[v].begin(), nb[v].end(), M.cols.begin() + M.rowptr[v]);
    M.diag[v] = M.rowptr[v] + int(std::lower_bound(nb[v].begin(), nb[v].end(), v) - nb[v].begin());
  }
  M.tetBlocks.resize(16 * (size_t)nt);
  for (int t = 0; t < nt; t++)
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++) {
        const int u = tets[4 * t + a], w = tets[4 * t + b];
        const int* beg = &M.cols[M.rowptr[u]];
        const int* end = &M.cols[M.rowptr[u + 1]];
        M.tetBlocks[16 * (size_t)t + 4 * a + b] = M.rowptr[u] + int(std::lower_bound(beg, end, w) - beg);
      }
}

// Per-tet F = Ds DmInv (TET_MESH.cpp:706-714), force
// -vol pFpx^T vec(P) (TET_MESH.cpp:736-747) and element Hessian
// pFpx^T (-vol clampedHessian) pFpx (TET_MESH_FASTER.cpp:95-103).
void elementTerms(const Mesh& M, const MaterialParams& mat, const double* disp, int t, double* F, double* U,
                  double* S, double* V, double* fe, double* He) {
  const int* v = &M.tets[4 * (size_t)t];
  double x[4][3];
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) x[a][i] = M.rest[3 * v[a] + i] + disp[3 * v[a] + i];
  double Ds[9];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 3; i++) Ds[i + 3 * a] = x[a + 1][i] - x[0][i];
  mul3(Ds, &M.DmInv[9 * (size_t)t], F);
  svd_rv(F, U, S, V);
  double P9[108];
  pFpx(&M.DmInv[9 * (size_t)t], P9);
  const double vol = M.vol[t];
  if (fe) {
    double P[9];
    PK1(mat, F, P);
    for (int c = 0; c < 12; c++) {
      double s = 0;
      for (int r = 0; r < 9; r++) s += P9[r + 9 * c] * P[r];
      fe[c] = -vol * s;
    }
  }
  if (He) {
    double H9[81], T[108];
    clampedHessian(mat, U, S, V, H9);
    for (int k = 0; k < 81; k++) H9[k] *= -vol;
    for (int c = 0; c < 12; c++)
      for (int r = 0; r < 9; r++) {
        double s = 0;
        for (int k = 0; k < 9; k++) s += H9[r + 9 * k] * P9[k + 9 * c];
        T[r + 9 * c] = s;
      }
    for (int c = 0; c < 12; c++)
      for (int r = 0; r < 12; r++) {
        double s = 0;
        for (int k = 0; k < 9; k++) s += P9[k + 9 * r] * T[k + 9 * c];
        He[r + 12 * c] = s;
      }
  }
}

// Deterministic chunked dot product (fixed summation tree, any thread count).
double dot(const std::vector<double>& a, const std::vector<double>& b) {
  const long n = (long)a.size();
  const long chunk = 4096;
  const long nc = (n + chunk - 1) / chunk;
  std::vector<double> part(nc);
#pragma omp parallel for schedule(static)
  for (long c = 0; c < nc; c++) {
    double s = 0;
    const long e = std::min(n, (c + 1) * chunk);
    for (long i = c * chunk; i < e; i++) s += a[i] * b[i];
    part[c] = s;
  }
  double s = 0;
  for (long c = 0; c < nc; c++) s += part[c];
  return s;
}

// ---------------------------------------------------------------------------
// Vertex-face self collisions (collision tets, VERTEX_FACE_SQRT_COLLISION).
// ---------------------------------------------------------------------------
typedef std::array<double, 3> V3;
inline V3 sub(const V3& a, const V3& b) { return {a[0] - b[0], a[1] - b[1], a[2] - b[2]}; }
inline V3 add(const V3& a, const V3& b) { return {a[0] + b[0], a[1] + b[1], a[2] + b[2]}; }
inline V3 mul(double s, const V3& a) { return {s * a[0], s * a[1], s * a[2]}; }
inline double dot3(const V3& a, const V3& b) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }
inline V3 cross3(const V3& a, const V3& b) {
  return {a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0]};
}
inline double norm3(const V3& a) { return std::sqrt(dot3(a, a)); }
inline V3 normalized(const V3& a) { return mul(1.0 / norm3(a), a); }

struct Collisions {
  bool on = false;
  bool ee = false;               // edge-edge self collisions
  std::vector<int> edges;        // 2 per surface edge, (lo, hi), ascending like a std::map
  std::vector<double> edgeArea;  // per surface edge: 1/3 of each adjacent triangle's rest area
  std::vector<int> edgeTri;      // 2 per surface edge: first two adjacent triangles (-1: none)
  std::vector<int> eePairs;      // per step: (edge, edge) pairs, surface edge indices
  double eps = 0.01, mu = 1.0, beta = 0.001;
  std::vector<int> tris;         // 3 per surface triangle, reference winding
  std::vector<int> surfVerts;    // ascending vertex ids
  std::vector<int> surfId;       // vertex -> index in surfVerts, or -1
  std::vector<int> nbr;          // 3 neighbouring triangles per triangle
  std::vector<double> restArea;  // per surface triangle
  std::vector<double> ringArea;  // per surface vertex
  // per step
  std::vector<int> pairs;        // (vertex, triangle) pairs
  std::vector<int> ctets;        // 4 per pair: vertex, face[2], face[1], face[0]
  std::vector<double> weight;    // rest face area + rest vertex one-ring area
  std::vector<double> f12, H12;  // per pair: -w grad (12), -w clamped Hessian (144, column major)
};

// Surface triangles in tet order with the reference winding
// (TET_MESH.cpp:294-350), surface vertices (567-590), triangle neighbours
// across edges (423-490) and rest areas (494-525).
void buildSurface(const Mesh& M, Collisions& C) {
  std::map<std::array<int, 3>, int> counts;
  auto faces = [&](int t, std::array<int, 3> f[4]) {
    const int* v = &M.tets[4 * (size_t)t];
    f[0] = {v[0], v[1], v[3]};
    f[1] = {v[0], v[2], v[1]};
    f[2] = {v[0], v[3], v[2]};
    f[3] = {v[1], v[2], v[3]};
  };
  for (int t = 0; t < M.nt; t++) {
    std::array<int, 3> f[4];
    faces(t, f);
    for (auto& x : f) {
      std::array<int, 3> s = x;
      std::sort(s.begin(), s.end());
      counts[s]++;
    }
  }
  C.tris.clear();
  for (int t = 0; t < M.nt; t++) {
    std::array<int, 3> f[4];
    faces(t, f);
    for (auto& x : f) {
      std::array<int, 3> s = x;
      std::sort(s.begin(), s.end());
      if (counts[s] < 2) C.tris.insert(C.tris.end(), x.begin(), x.end());
    }
  }
  const int ntri = (int)C.tris.size() / 3;
  std::vector<char> on(M.nv, 0);
  for (int k : C.tris) on[k] = 1;
  C.surfVerts.clear();
  C.surfId.assign(M.nv, -1);
  for (int v = 0; v < M.nv; v++)
    if (on[v]) {
      C.surfId[v] = (int)C.surfVerts.size();
      C.surfVerts.push_back(v);
    }
  std::multimap<std::pair<int, int>, int> edges;
  for (int i = 0; i < ntri; i++)
    for (int j = 0; j < 3; j++) {
      int a = C.tris[3 * i + j], b = C.tris[3 * i + (j + 1) % 3];
      if (a > b) std::swap(a, b);
      edges.insert({{a, b}, i});
    }
  C.nbr.assign(3 * (size_t)ntri, -1);
  for (int i = 0; i < ntri; i++)
    for (int j = 0; j < 3; j++) {
      int a = C.tris[3 * i + j], b = C.tris[3 * i + (j + 1) % 3];
      if (a > b) std::swap(a, b);
      auto range = edges.equal_range({a, b});
      for (auto it = range.first; it != range.second; ++it)
        if (it->second != i) C.nbr[3 * i + j] = it->second;
    }
  auto restV = [&](int v) { return V3{M.rest[3 * v], M.rest[3 * v + 1], M.rest[3 * v + 2]}; };
  C.restArea.resize(ntri);
  C.ringArea.assign(C.surfVerts.size(), 0.0);
  for (int i = 0; i < ntri; i++) {
    const V3 a = restV(C.tris[3 * i]), b = restV(C.tris[3 * i + 1]), c = restV(C.tris[3 * i + 2]);
    C.restArea[i] = 0.5 * norm3(cross3(sub(b, a), sub(c, a)));
    for (int j = 0; j < 3; j++) C.ringArea[C.surfId[C.tris[3 * i + j]]] += (1.0 / 3.0) * C.restArea[i];
  }
}

// TET_MESH::pointProjectsInsideTriangle (TET_MESH.cpp:1296-1317) and the
// barycentric test it shares with pointTriangleDistance.
bool projectsInside(const V3& v0, const V3& v1, const V3& v2, const V3& v) {
  const V3 n = cross3(sub(v1, v0), sub(v2, v0));
  const double nn = dot3(n, n);
  const double b0 = dot3(n, cross3(sub(v2, v1), sub(v, v1))) / nn;
  const double b1 = dot3(n, cross3(sub(v0, v2), sub(v, v2))) / nn;
  const double b2 = dot3(n, cross3(sub(v1, v0), sub(v, v0))) / nn;
  return std::fabs(b0) + std::fabs(b1) + std::fabs(b2) - 1.0 < 1e-8;
}

// TET_MESH::pointTriangleDistance (TET_MESH.cpp:1322-1388)
double pointTriangleDistance(const V3& v0, const V3& v1, const V3& v2, const V3& v) {
  const V3 e1 = sub(v1, v0), e2 = sub(v2, v0);
  const V3 n = cross3(e1, e2);
  if (projectsInside(v0, v1, v2, v)) return std::fabs(dot3(mul(1.0 / norm3(n), n), sub(v, v0)));
  const V3 e3 = sub(v2, v1), ev = sub(v, v0), ev3 = sub(v, v1);
  const double big = std::numeric_limits<float>::max();
  double ed[3] = {big, big, big};
  const double l1 = norm3(e1), l2 = norm3(e2), l3 = norm3(e3);
  const double d1 = dot3(mul(1.0 / l1, e1), ev);
  if (d1 > 0.0 && d1 < l1) ed[0] = norm3(sub(v, add(v0, mul(d1, mul(1.0 / l1, e1)))));
  const double d2 = dot3(mul(1.0 / l2, e2), ev);
  if (d2 > 0.0 && d2 < l2) ed[1] = norm3(sub(v, add(v0, mul(d2, mul(1.0 / l2, e2)))));
  const double d3 = dot3(mul(1.0 / l3, e3), ev3);
  if (d3 > 0.0 && d3 < l3) ed[2] = norm3(sub(v, add(v1, mul(d3, mul(1.0 / l3, e3)))));
  const double vmin = std::min(norm3(sub(v, v0)), std::min(norm3(sub(v, v1)), norm3(sub(v, v2))));
  const double emin = std::min(ed[0], std::min(ed[1], ed[2]));
  return vmin < emin ? vmin : emin;
}

// VERTEX_FACE_SQRT_COLLISION on a collision tet (v0 = vertex, v1..v3 = face):
// gradient (VERTEX_FACE_SQRT_COLLISION.cpp:140-181) and the eigenvalue-clamped
// Hessian (185-219 with clampEigenvalues, MATRIX_UTIL.cpp:116-127), with the
// inside barycentric coordinates of COLLISION_UTIL.cpp:314-502.
void vfSqrt(const V3 v[4], double mu, double eps, double* g, double* H);

void jacobiEigen(int n, std::vector<double>& a, std::vector<double>& q);

void vfBarycentric(const V3 v[4], double bary[3]) {
  const V3 e1 = sub(v[2], v[1]), e2 = sub(v[3], v[1]);
  const V3 n = cross3(e1, e2);
  const V3 nh = mul(1.0 / norm3(n), n);
  const V3 p = sub(v[0], mul(dot3(nh, sub(v[0], v[1])), nh));
  const double nn = dot3(n, n);
  bary[0] = dot3(n, cross3(sub(v[3], v[2]), sub(p, v[2]))) / nn;
  bary[1] = dot3(n, cross3(sub(v[1], v[3]), sub(p, v[3]))) / nn;
  bary[2] = dot3(n, cross3(sub(v[2], v[1]), sub(p, v[1]))) / nn;
  if (bary[0] >= 0.0 && bary[1] >= 0.0 && bary[2] >= 0.0) return;
  auto lineDist = [](const V3& p0, const V3& p1, const V3& p2) {
    const V3 e0 = sub(p0, p1), e = sub(p2, p1);
    const double l = norm3(e);
    const double proj = dot3(e0, mul(1.0 / l, e));
    if (proj > 0.0 && proj < l) return norm3(sub(e0, mul(proj, mul(1.0 / l, e))));
    const double a = norm3(sub(p0, p1)), b = norm3(sub(p0, p2));
    return a < b ? a : b;
  };
  auto lerp = [](const V3& p0, const V3& p1, const V3& p2, double out[2]) {
    const V3 e0 = sub(p0, p1), e = sub(p2, p1);
    const double l = norm3(e);
    const double proj = dot3(e0, mul(1.0 / l, e));
    if (proj < 0.0) { out[0] = 1.0; out[1] = 0.0; return; }
    if (proj >= l) { out[0] = 0.0; out[1] = 1.0; return; }
    const double r = proj / l;
    out[0] = 1.0 - r;
    out[1] = r;
  };
  const double d12 = lineDist(v[0], v[1], v[2]), d23 = lineDist(v[0], v[2], v[3]), d31 = lineDist(v[0], v[3], v[1]);
  double l[2];
  if (d12 <= d23 && d12 <= d31) {
    lerp(v[0], v[1], v[2], l);
    bary[0] = l[0]; bary[1] = l[1]; bary[2] = 0.0;
  } else if (d23 <= d12 && d23 <= d31) {
    lerp(v[0], v[2], v[3], l);
    bary[0] = 0.0; bary[1] = l[0]; bary[2] = l[1];
  } else {
    lerp(v[0], v[3], v[1], l);
    bary[0] = l[1]; bary[1] = 0.0; bary[2] = l[0];
  }
}

void vfSqrt(const V3 v[4], double mu, double eps, double* g, double* H) {
  double bary[3];
  vfBarycentric(v, bary);
  // reverse(): n = e2 x e0 with e0 = v3 - v2, e1 = v0 - v2, e2 = v1 - v2
  const V3 e0 = sub(v[3], v[2]), e1 = sub(v[0], v[2]), e2 = sub(v[1], v[2]);
  const V3 n = normalized(cross3(e2, e0));
  const bool reversal = dot3(n, e1) < 0;
  const V3 xs = add(add(mul(bary[0], v[1]), mul(bary[1], v[2])), mul(bary[2], v[3]));
  const V3 t = sub(v[0], xs);
  const double tt = dot3(t, t), tm = std::sqrt(tt);
  const double spring = reversal ? tm + eps : tm - eps;
  std::fill(g, g + 12, 0.0);
  std::fill(H, H + 144, 0.0);
  if (std::fabs(tm) <= 1e-8 || std::fabs(tt) < 1e-8) return;
  const double c[4] = {1.0, -bary[0], -bary[1], -bary[2]};  // tDiffPartial (MCADAMS_COLLISION.cpp:238-248)
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++) g[3 * a + i] = 2.0 * mu * spring * (1.0 / tm) * c[a] * t[i];
  // hessian = 2 mu ((1/tt - spring/(tt tm)) (D^T t)(D^T t)^T + (spring/tm) D^T D)
  std::vector<double> A(144);
  const double k1 = 1.0 / tt - spring / (tt * tm), k2 = spring / tm;
  for (int a = 0; a < 4; a++)
    for (int i = 0; i < 3; i++)
      for (int b = 0; b < 4; b++)
        for (int j = 0; j < 3; j++) {
          const double pp = (c[a] * t[i]) * (c[b] * t[j]);
          const double dd = (i == j) ? c[a] * c[b] : 0.0;
          A[(3 * a + i) + 12 * (3 * b + j)] = 2.0 * mu * (k1 * pp + k2 * dd);
        }
  std::vector<double> Q;
  jacobiEigen(12, A, Q);  // A -> diagonal, Q eigenvectors (columns)
  for (int r = 0; r < 12; r++)
    for (int cc = 0; cc < 12; cc++) {
      double s = 0;
      for (int k = 0; k < 12; k++) {
        const double lam = A[k + 12 * k] > 0.0 ? A[k + 12 * k] : 0.0;
        s += Q[r + 12 * k] * lam * Q[cc + 12 * k];
      }
      H[r + 12 * cc] = s;
    }
}

// Cyclic Jacobi eigen-decomposition of a symmetric n x n matrix (column
// major, overwritten by its eigenvalues on the diagonal); Q = eigenvectors.
// Stands in for Eigen::SelfAdjointEigenSolver (MATRIX_UTIL.cpp:116-127).
void jacobiEigen(int n, std::vector<double>& a, std::vector<double>& q) {
  q.assign((size_t)n * n, 0.0);
  for (int i = 0; i < n; i++) q[i + n * i] = 1.0;
  for (int sweep = 0; sweep < 100; sweep++) {
    double off = 0, diag = 0;
    for (int j = 0; j < n; j++)
      for (int i = 0; i < n; i++) (i == j ? diag : off) += std::fabs(a[i + n * j]);
    if (off == 0.0 || off <= 1e-15 * diag) break;
    for (int p = 0; p < n; p++)
      for (int k = p + 1; k < n; k++) {
        const double apk = a[p + n * k];
        if (apk == 0.0) continue;
        const double theta = (a[k + n * k] - a[p + n * p]) / (2.0 * apk);
        const double t = (theta >= 0 ? 1.0 : -1.0) / (std::fabs(theta) + std::sqrt(theta * theta + 1.0));
        const double c = 1.0 / std::sqrt(t * t + 1.0), s = t * c;
        for (int m = 0; m < n; m++) {
          const double amp = a[m + n * p], amk = a[m + n * k];
          a[m + n * p] = c * amp - s * amk;
          a[m + n * k] = s * amp + c * amk;
        }
        for (int m = 0; m < n; m++) {
          const double apm = a[p + n * m], akm = a[k + n * m];
          a[p + n * m] = c * apm - s * akm;
          a[k + n * m] = s * apm + c * akm;
        }
        for (int m = 0; m < n; m++) {
          const double qmp = q[m + n * p], qmk = q[m + n * k];
          q[m + n * p] = c * qmp - s * qmk;
          q[m + n * k] = s * qmp + c * qmk;
        }
      }
  }
}

struct Sim {
  Mesh M;
  MaterialParams mat;
  Collisions coll;
  std::vector<int> pinned;
  std::vector<double> pinTarget;  // 3 per pinned vertex
  std::vector<unsigned char> free;  // per vertex: 1 = free, 0 = pinned (S block = I or 0)
  double density = 1.0, dt = 1.0 / 60.0;
  double gravity[3] = {0, 0, 0};
  double tol = 1e-8;
  int maxit = 1000;
  int precond = 0;  // 0 = scalar Jacobi (Eigen DiagonalPreconditioner), 1 = 3x3 block Jacobi
  std::vector<double> x, v, fext;
  std::vector<double> K, A, R, He, fe;
  std::vector<double> collDiag;  // per vertex 3x3: collision part of LHS's diagonal
  double collScale = 0.0;        // -(dt beta + dt^2): collision Hessian's weight in A
  int lastIters = 0;
  double lastErr = 0;
  // integrator: 0 BACKWARD_EULER_VELOCITY, 1 BACKWARD_EULER_POSITION (Rayleigh
  // damped, C = alpha M + beta K0 with K0 the clamped Hessian at rest)
  int integrator = 0;
  double rayAlpha = 0.01, rayBeta = 0.01;  // BACKWARD_EULER_POSITION.cpp:53-54
  std::vector<double> K0;
  // NEWMARK (integrator 2): acceleration state and the Newton loop's limits
  // (NEWMARK.cpp:38-43)
  std::vector<double> acc;
  int maxNewton = 10;
  double newtonEps = 1e-7;
  double greenMu = 0.0;  // NEWMARK with GREEN_DAMPING(mu): the energy-damped solve
  int lastNewton = 0;
};

// Vertex-face detection at the current displacement: inverted vertices
// (TET_MESH.cpp:2450-2475), then per surface vertex in ascending order the
// triangles that pass the narrow phase of
// TET_MESH_FASTER::computeVertexFaceCollisions (TET_MESH_FASTER.cpp:248-334),
// brute force instead of the AABB broad phase, in ascending triangle order,
// and the collision tets of buildVertexFaceCollisionTets (TET_MESH.cpp:1785-1826).
void vfDetect(Sim& s) {
  const Mesh& M = s.M;
  Collisions& C = s.coll;
  auto pos = [&](int v) {
    return V3{M.rest[3 * v] + s.x[3 * v], M.rest[3 * v + 1] + s.x[3 * v + 1], M.rest[3 * v + 2] + s.x[3 * v + 2]};
  };
  std::vector<char> inverted(M.nv, 0);
  for (int t = 0; t < M.nt; t++) {
    const int* tv = &M.tets[4 * (size_t)t];
    const V3 x0 = pos(tv[0]);
    double Ds[9], F[9];
    for (int a = 0; a < 3; a++) {
      const V3 d = sub(pos(tv[a + 1]), x0);
      for (int i = 0; i < 3; i++) Ds[i + 3 * a] = d[i];
    }
    mul3(Ds, &M.DmInv[9 * (size_t)t], F);
    if (det3(F) > 0.0) continue;
    for (int a = 0; a < 4; a++) inverted[tv[a]] = 1;
  }
  const int ntri = (int)C.tris.size() / 3;
  std::vector<char> degenerate(ntri), allInverted(ntri);
  for (int f = 0; f < ntri; f++) {
    const int* t = &C.tris[3 * f];
    const double area = 0.5 * norm3(cross3(sub(pos(t[1]), pos(t[0])), sub(pos(t[2]), pos(t[0]))));
    degenerate[f] = area / C.restArea[f] < 1e-4;  // surfaceTriangleIsDegenerate (TET_MESH.cpp:2421-2445)
    allInverted[f] = inverted[t[0]] && inverted[t[1]] && inverted[t[2]];
  }
  C.pairs.clear();
  for (int v : C.surfVerts) {
    if (inverted[v]) continue;
    const V3 p = pos(v);
    for (int f = 0; f < ntri; f++) {
      const int* t = &C.tris[3 * f];
      if (degenerate[f] || allInverted[f]) continue;
      if (t[0] == v || t[1] == v || t[2] == v) continue;
      const V3 a = pos(t[0]), b = pos(t[1]), c = pos(t[2]);
      if (!(pointTriangleDistance(a, b, c, p) < C.eps)) continue;
      bool hit = projectsInside(a, b, c, p);
      if (!hit) {  // insideCollisionCell (TET_MESH.cpp:1396-1437)
        const V3 vv[3] = {a, b, c};
        const V3 n = normalized(cross3(sub(b, a), sub(c, a)));
        hit = true;
        for (int k = 0; k < 3 && hit; k++) {
          const int* tn = &C.tris[3 * C.nbr[3 * f + k]];
          const V3 na = pos(tn[0]), nb = pos(tn[1]), nc = pos(tn[2]);
          const V3 nn = normalized(cross3(sub(nb, na), sub(nc, na)));
          const V3 ne = normalized(add(nn, n));
          const V3 eij = sub(vv[(k + 1) % 3], vv[k]);
          const V3 neb = normalized(cross3(ne, eij));
          if (dot3(neb, sub(p, vv[k])) < 0.0) hit = false;
        }
      }
      if (hit) {
        C.pairs.push_back(v);
        C.pairs.push_back(f);
      }
    }
  }
  const int np = (int)C.pairs.size() / 2;
  C.ctets.resize(4 * (size_t)np);
  C.weight.resize(np);
  for (int k = 0; k < np; k++) {
    const int v = C.pairs[2 * k], f = C.pairs[2 * k + 1];
    const int* t = &C.tris[3 * f];
    C.ctets[4 * k] = v;
    C.ctets[4 * k + 1] = t[2];
    C.ctets[4 * k + 2] = t[1];
    C.ctets[4 * k + 3] = t[0];
    C.weight[k] = C.restArea[f] + C.ringArea[C.surfId[v]];
  }
}

// Collision forces and clamped Hessians per collision tet
// (TET_MESH.cpp:1831-1877, 2045-2088), both scaled by -weight.
void vfResponse(Sim& s) {
  const Mesh& M = s.M;
  Collisions& C = s.coll;
  const int np = (int)C.weight.size();
  C.f12.assign(12 * (size_t)np, 0.0);
  C.H12.assign(144 * (size_t)np, 0.0);
#pragma omp parallel for schedule(static)
  for (int k = 0; k < np; k++) {
    V3 v[4];
    for (int a = 0; a < 4; a++) {
      const int id = C.ctets[4 * k + a];
      v[a] = V3{M.rest[3 * id] + s.x[3 * id], M.rest[3 * id + 1] + s.x[3 * id + 1],
                M.rest[3 * id + 2] + s.x[3 * id + 2]};
    }
    double g[12], H[144];
    vfSqrt(v, C.mu, C.eps, g, H);
    for (int i = 0; i < 12; i++) C.f12[12 * (size_t)k + i] = -C.weight[k] * g[i];
    for (int i = 0; i < 144; i++) C.H12[144 * (size_t)k + i] = -C.weight[k] * H[i];
  }
}

// ---------------------------------------------------------------------------
// Edge-edge self collisions (EDGE_SQRT_COLLISION on surface edge pairs).
// ---------------------------------------------------------------------------
// Surface edges in std::map order of (lo, hi) (TET_MESH::computeSurfaceEdges,
// TET_MESH.cpp:595-630), each edge's rest area (a third of each adjacent
// surface triangle's rest area, TET_MESH.cpp:530-562) and its first two
// adjacent triangles in triangle order (computeSurfaceEdgeTriangleNeighbors,
// TET_MESH.cpp:356-412).
void buildEdges(Collisions& C) {
  const int ntri = (int)C.tris.size() / 3;
  std::vector<std::pair<int, int>> e;
  for (int t = 0; t < ntri; t++)
    for (int j = 0; j < 3; j++) {
      const int a = C.tris[3 * t + j], b = C.tris[3 * t + (j + 1) % 3];
      e.push_back({std::min(a, b), std::max(a, b)});
    }
  std::sort(e.begin(), e.end());
  e.erase(std::unique(e.begin(), e.end()), e.end());
  const int ne = (int)e.size();
  C.edges.resize(2 * ne);
  for (int k = 0; k < ne; k++) {
    C.edges[2 * k] = e[k].first;
    C.edges[2 * k + 1] = e[k].second;
  }
  C.edgeArea.assign(ne, 0.0);
  C.edgeTri.assign(2 * ne, -1);
  for (int t = 0; t < ntri; t++)
    for (int j = 0; j < 3; j++) {
      const int a = C.tris[3 * t + j], b = C.tris[3 * t + (j + 1) % 3];
      const int k = (int)(std::lower_bound(e.begin(), e.end(), std::make_pair(std::min(a, b), std::max(a, b))) -
                          e.begin());
      C.edgeArea[k] += C.restArea[t] / 3.0;
      if (C.edgeTri[2 * k] < 0) C.edgeTri[2 * k] = t;
      else if (C.edgeTri[2 * k + 1] < 0) C.edgeTri[2 * k + 1] = t;
    }
}

// Closest points of two segments, restating the published routine the
// reference uses (Rhodes, "Fast, Robust Intersection of 3D Line Segments",
// Game Programming Gems II; LINE_INTERSECT.cpp), with its tolerances: the
// call passes 1e-8 both as the parallel/degenerate tolerance and where the
// helpers take a squared tolerance.
namespace segseg {
const double kTol = 1e-8;
inline bool outside01(double a) { return a < 0.0 || a > 1.0; }
inline double clamp01(double a) { return std::max(0.0, std::min(1.0, a)); }
// nearest point to q on the line/segment p + s L
void nearestOnSegment(const V3& p, const V3& L, const V3& q, bool infinite, V3& out, double& param) {
  const double D = dot3(L, L);
  if (D < kTol) {
    out = p;
    return;
  }
  param = dot3(L, sub(q, p)) / D;
  if (!infinite) param = clamp01(param);
  out = add(p, mul(param, L));
}
void parallel(const V3& a1, const V3& a2, const V3& La, const V3& b1, const V3& b2, const V3& Lb, V3& pa, V3& pb) {
  double s0 = 0.0, s1 = 0.0, tmp = 0.0;
  nearestOnSegment(a1, La, b1, true, pa, s0);
  V3 scratch;
  nearestOnSegment(a1, La, b2, true, scratch, s1);
  if (s0 < 0.0 && s1 < 0.0) {
    pa = a1;
    pb = s0 < s1 ? b2 : b1;
  } else if (s0 > 1.0 && s1 > 1.0) {
    pa = a2;
    pb = s0 < s1 ? b1 : b2;
  } else {
    tmp = 0.5 * (clamp01(s0) + clamp01(s1));
    pa = add(a1, mul(tmp, La));
    nearestOnSegment(b1, Lb, pa, true, pb, tmp);
  }
}
void adjust(const V3& a1, const V3& La, const V3& b1, const V3& Lb, double s, double t, V3& pa, V3& pb) {
  if (outside01(s) && outside01(t)) {
    s = clamp01(s);
    pa = add(a1, mul(s, La));
    nearestOnSegment(b1, Lb, pa, true, pb, t);
    if (outside01(t)) {
      t = clamp01(t);
      pb = add(b1, mul(t, Lb));
      nearestOnSegment(a1, La, pb, false, pa, s);
      nearestOnSegment(b1, Lb, pa, false, pb, t);
    }
  } else if (outside01(s)) {
    s = clamp01(s);
    pa = add(a1, mul(s, La));
    nearestOnSegment(b1, Lb, pa, false, pb, t);
  } else if (outside01(t)) {
    t = clamp01(t);
    pb = add(b1, mul(t, Lb));
    nearestOnSegment(a1, La, pb, false, pa, s);
  }
}
void closest(const V3& a1, const V3& a2, const V3& b1, const V3& b2, V3& pa, V3& pb) {
  const V3 La = sub(a2, a1), Lb = sub(b2, b1);
  const double L11 = dot3(La, La), L22 = dot3(Lb, Lb), tol2 = kTol * kTol;
  double tmp = 0.0;
  if (L11 < tol2) {
    pa = a1;
    nearestOnSegment(b1, Lb, a1, false, pb, tmp);
  } else if (L22 < tol2) {
    pb = b1;
    nearestOnSegment(a1, La, b1, false, pa, tmp);
  } else {
    const V3 AB = sub(b1, a1);
    const double L12 = -dot3(La, Lb);
    const double det = L11 * L22 - L12 * L12;
    if (std::fabs(det) < kTol) {
      parallel(a1, a2, La, b1, b2, Lb, pa, pb);
    } else {
      const double ra = dot3(La, AB);
      const double rb = -dot3(Lb, AB);
      const double t = (L11 * rb - ra * L12) / det;
      const double s = (ra - L12 * t) / L11;
      pa = add(a1, mul(s, La));
      pb = add(b1, mul(t, Lb));
      if (outside01(s) || outside01(t)) adjust(a1, La, b1, Lb, s, t, pa, pb);
    }
  }
}
}  // namespace segseg

// faceEdgeIntersection (COLLISION_UTIL.cpp:577-613): does the ray from e0
// along e1 - e0 cross triangle (a, b, c) before reaching e1?
bool faceEdgeCross(const V3& a, const V3& b, const V3& c, const V3& e0, const V3& e1) {
  const V3 ed = sub(e1, e0);
  const V3 dir = normalized(ed);
  const V3 n = normalized(cross3(sub(b, a), sub(c, a)));
  const double denom = dot3(dir, n);
  if (std::fabs(denom) <= 0.0) return false;
  const double t = dot3(sub(a, e0), n) / denom;
  if (t < 0) return false;
  const V3 h = add(e0, mul(t, dir));
  if (dot3(n, cross3(sub(b, a), sub(h, a))) < 0) return false;
  if (dot3(n, cross3(sub(c, b), sub(h, b))) < 0) return false;
  if (dot3(n, cross3(sub(a, c), sub(h, c))) < 0) return false;
  return t < norm3(ed);
}

// TET_MESH_FASTER::computeEdgeEdgeCollisions (TET_MESH_FASTER.cpp:340-500):
// for every surface edge x the closest non-adjacent surface edge y >= x whose
// closest points lie inside both edges (parameters in [1e-4, 1 - 1e-4]),
// ties to the later one; kept when no endpoint pair is a surface edge (the
// one-ring test, TET_MESH.cpp:2145-2155) and the distance is below eps.  Then
// EDGE_SQRT_COLLISION (EDGE_SQRT_COLLISION.cpp:40-231) on the pair, negated
// when the edge crosses a triangle next to the other edge:
//   diff = (b0 v2 + b1 v3) - (a0 v0 + a1 v1), r = |diff|, n = diff / r,
//   c = (-a0, -a1, b0, b1), spring = r - eps (negated: r + eps),
//   grad = 2 mu spring (c (x) n), clamped Hessian = (c c^T) (x) G with
//   G = 2 mu (n n^T + max(spring / r, 0) (I - n n^T)) -- the 12x12
//   eigenvalue clamp of (c c^T) (x) G3 clamps G3 alone;
//   zero when r < 1e-7.  Forces -w grad, Hessians -w H, w = the two edges'
//   rest areas summed.
void eeCollisions(Sim& s) {
  const Mesh& M = s.M;
  Collisions& C = s.coll;
  if (C.edges.empty()) buildEdges(C);
  const int ne = (int)C.edges.size() / 2;
  auto pos = [&](int id) {
    return V3{M.rest[3 * id] + s.x[3 * id], M.rest[3 * id + 1] + s.x[3 * id + 1], M.rest[3 * id + 2] + s.x[3 * id + 2]};
  };
  std::vector<std::pair<int, int>> adj;
  for (int k = 0; k < ne; k++) {
    adj.push_back({C.edges[2 * k], C.edges[2 * k + 1]});
    adj.push_back({C.edges[2 * k + 1], C.edges[2 * k]});
  }
  std::sort(adj.begin(), adj.end());
  auto adjacent = [&](int a, int b) { return std::binary_search(adj.begin(), adj.end(), std::make_pair(a, b)); };
  const double farAway = (double)FLT_MAX;
  // boxes for a cheap prefilter: an edge whose eps-inflated box misses x's
  // box is farther than eps and can neither be kept nor be x's partner in a
  // kept pair, so skipping it leaves the pairs unchanged
  std::vector<double> box(6 * (size_t)ne);
  for (int k = 0; k < ne; k++) {
    const V3 p = pos(C.edges[2 * k]), q = pos(C.edges[2 * k + 1]);
    for (int i = 0; i < 3; i++) {
      box[6 * k + i] = std::min(p[i], q[i]);
      box[6 * k + 3 + i] = std::max(p[i], q[i]);
    }
  }
  struct Hit {
    int best;
    double d, a[2], b[2];
  };
  std::vector<Hit> hits(ne);
#pragma omp parallel for schedule(dynamic, 64)
  for (int x = 0; x < ne; x++) {
    const int o0 = C.edges[2 * x], o1 = C.edges[2 * x + 1];
    const V3 v0 = pos(o0), v1 = pos(o1);
    int best = -1;
    double bestD = farAway, ba[2] = {-1, -1}, bb[2] = {-1, -1};
    for (int y = x; y < ne; y++) {
      const int i0 = C.edges[2 * y], i1 = C.edges[2 * y + 1];
      if (o0 == i0 || o0 == i1 || o1 == i0 || o1 == i1) continue;
      bool apart = false;
      for (int i = 0; i < 3; i++)
        apart = apart || box[6 * y + i] - C.eps > box[6 * x + 3 + i] || box[6 * y + 3 + i] + C.eps < box[6 * x + i];
      if (apart) continue;
      const V3 v2 = pos(i0), v3 = pos(i1);
      V3 po, pi;
      segseg::closest(v0, v1, v2, v3, po, pi);
      const double d = norm3(sub(pi, po));
      if (d > bestD) continue;
      double a[2], b[2];
      a[1] = norm3(sub(po, v0)) / norm3(sub(v1, v0));
      a[0] = 1.0 - a[1];
      b[1] = norm3(sub(pi, v2)) / norm3(sub(v3, v2));
      b[0] = 1.0 - b[1];
      const double skip = 1e-4;
      if (a[0] < skip || a[0] > 1.0 - skip || a[1] < skip || a[1] > 1.0 - skip) continue;
      if (b[0] < skip || b[0] > 1.0 - skip || b[1] < skip || b[1] > 1.0 - skip) continue;
      bestD = d;
      best = y;
      ba[0] = a[0], ba[1] = a[1], bb[0] = b[0], bb[1] = b[1];
    }
    hits[x] = Hit{best, bestD, {ba[0], ba[1]}, {bb[0], bb[1]}};
  }
  for (int x = 0; x < ne; x++) {
    const int o0 = C.edges[2 * x], o1 = C.edges[2 * x + 1];
    const V3 v0 = pos(o0), v1 = pos(o1);
    const int best = hits[x].best;
    const double bestD = hits[x].d, ba[2] = {hits[x].a[0], hits[x].a[1]}, bb[2] = {hits[x].b[0], hits[x].b[1]};
    if (best < 0) continue;
    const int i0 = C.edges[2 * best], i1 = C.edges[2 * best + 1];
    if (adjacent(o0, i0) || adjacent(o0, i1) || adjacent(o1, i0) || adjacent(o1, i1)) continue;
    if (!(bestD < C.eps)) continue;
    // penetration: the outer edge through a triangle next to the inner edge
    bool crossing = false;
    for (int q = 0; q < 2; q++) {
      const int t = C.edgeTri[2 * best + q];
      if (t < 0) continue;
      const bool hit = faceEdgeCross(pos(C.tris[3 * t]), pos(C.tris[3 * t + 1]), pos(C.tris[3 * t + 2]), v0, v1);
      crossing = crossing || hit;
    }
    const double w = C.edgeArea[x] + C.edgeArea[best];
    const int ids[4] = {o0, o1, i0, i1};
    const double cv[4] = {-ba[0], -ba[1], bb[0], bb[1]};
    V3 diff = {0, 0, 0};
    for (int a = 0; a < 4; a++) diff = add(diff, mul(cv[a], pos(ids[a])));
    const double r = norm3(diff);
    const size_t k = C.weight.size();
    C.eePairs.push_back(x);
    C.eePairs.push_back(best);
    for (int a = 0; a < 4; a++) C.ctets.push_back(ids[a]);
    C.weight.push_back(w);
    C.f12.resize(12 * (k + 1), 0.0);
    C.H12.resize(144 * (k + 1), 0.0);
    if (r < 1e-7) continue;
    const V3 n = mul(1.0 / r, diff);
    const double spring = crossing ? r + C.eps : r - C.eps;
    const double k2 = std::max(spring / r, 0.0);
    double G[9];
    for (int i = 0; i < 3; i++)
      for (int j = 0; j < 3; j++) G[i + 3 * j] = 2.0 * C.mu * ((1.0 - k2) * n[i] * n[j] + (i == j ? k2 : 0.0));
    for (int a = 0; a < 4; a++)
      for (int i = 0; i < 3; i++) C.f12[12 * k + 3 * a + i] = -w * (2.0 * C.mu * spring * cv[a] * n[i]);
    for (int a = 0; a < 4; a++)
      for (int b = 0; b < 4; b++)
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++)
            C.H12[144 * k + (3 * a + i) + 12 * (3 * b + j)] = -w * cv[a] * cv[b] * G[i + 3 * j];
  }
}

// K = sum of element Hessians per block, gathered per row in ascending tet
// order like TET_MESH_FASTER's _hessianGathers (TET_MESH_FASTER.cpp:113-131);
// R = sum of element forces per vertex in ascending tet order
// (TET_MESH.cpp:756-767).
void assemble(Sim& s) {
  const Mesh& M = s.M;
  const int nt = M.nt, nv = M.nv;
  s.He.resize(144 * (size_t)nt);
  s.fe.resize(12 * (size_t)nt);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nt; t++) {
    double F[9], U[9], S[3], V[9];
    elementTerms(M, s.mat, s.x.data(), t, F, U, S, V, &s.fe[12 * (size_t)t], &s.He[144 * (size_t)t]);
  }
  s.K.assign(9 * (size_t)M.rowptr[nv], 0.0);
  s.R.assign(3 * (size_t)nv, 0.0);
#pragma omp parallel for schedule(static)
  for (int u = 0; u < nv; u++) {
    for (int k = M.vtxptr[u]; k < M.vtxptr[u + 1]; k++) {
      const int t = M.vtxinc[k] / 4, a = M.vtxinc[k] % 4;
      const double* H = &s.He[144 * (size_t)t];
      for (int i = 0; i < 3; i++) s.R[3 * u + i] += s.fe[12 * (size_t)t + 3 * a + i];
      for (int b = 0; b < 4; b++) {
        double* blk = &s.K[9 * (size_t)M.tetBlocks[16 * (size_t)t + 4 * a + b]];
        for (int c = 0; c < 3; c++)
          for (int r = 0; r < 3; r++) blk[r + 3 * c] += H[(3 * a + r) + 12 * (3 * b + c)];
      }
    }
  }
}

// y = LHS x with LHS = S A S + (I - S), S = diag(free) per vertex
// (BACKWARD_EULER_VELOCITY.cpp:170); A's blocks in `A`.
void applyLHS(const Sim& s, const std::vector<double>& A, const std::vector<double>& x, std::vector<double>& y) {
  const Mesh& M = s.M;
#pragma omp parallel for schedule(static)
  for (int u = 0; u < M.nv; u++) {
    if (!s.free[u]) {
      for (int i = 0; i < 3; i++) y[3 * u + i] = x[3 * u + i];
      continue;
    }
    for (int i = 0; i < 3; i++) {
      double acc = 0;
      for (int k = M.rowptr[u]; k < M.rowptr[u + 1]; k++) {
        const int w = M.cols[k];
        if (!s.free[w]) continue;
        const double* blk = &A[9 * (size_t)k];
        for (int c = 0; c < 3; c++) acc += blk[i + 3 * c] * x[3 * w + c];
      }
      y[3 * u + i] = acc;
    }
  }
  // collision tets: y += S (-(dt beta + dt^2) H_coll) S x, in pair order
  const Collisions& C = s.coll;
  for (size_t k = 0; k < C.weight.size(); k++) {
    const double* H = &C.H12[144 * k];
    for (int a = 0; a < 4; a++) {
      const int u = C.ctets[4 * k + a];
      if (!s.free[u]) continue;
      for (int b = 0; b < 4; b++) {
        const int w = C.ctets[4 * k + b];
        if (!s.free[w]) continue;
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) y[3 * u + i] += s.collScale * H[(3 * a + i) + 12 * (3 * b + j)] * x[3 * w + j];
      }
    }
  }
}

// Preconditioned CG restating Eigen's conjugate_gradient
// (ext/eigen-3.3.7/Eigen/src/IterativeLinearSolvers/ConjugateGradient.h:28-90)
// with x0 = 0 (ConjugateGradient.h:236) and the Jacobi preconditioner
// (BasicPreconditioners.h:67-75); precond = 1 swaps in 3x3 block Jacobi.
void pcg(Sim& s, const std::vector<double>& A, const std::vector<double>& rhs, std::vector<double>& x) {
  const Mesh& M = s.M;
  const size_t n = 3 * (size_t)M.nv;
  x.assign(n, 0.0);
  std::vector<double> r(rhs), p(n), z(n), tmp(n), inv(9 * (size_t)M.nv, 0.0);
  // preconditioner from LHS's diagonal (pinned blocks are identity)
  for (int u = 0; u < M.nv; u++) {
    double* B = &inv[9 * (size_t)u];
    if (!s.free[u]) {
      B[0] = B[4] = B[8] = 1.0;
      continue;
    }
    double D[9];
    for (int k = 0; k < 9; k++)
      D[k] = A[9 * (size_t)M.diag[u] + k] + (s.collDiag.empty() ? 0.0 : s.collDiag[9 * (size_t)u + k]);
    if (s.precond == 1) {
      inv3(D, B);
    } else {
      for (int i = 0; i < 3; i++) B[4 * i] = D[4 * i] != 0.0 ? 1.0 / D[4 * i] : 1.0;
    }
  }
  auto applyPrec = [&](const std::vector<double>& in, std::vector<double>& out) {
#pragma omp parallel for schedule(static)
    for (int u = 0; u < M.nv; u++) {
      const double* B = &inv[9 * (size_t)u];
      for (int i = 0; i < 3; i++) {
        if (s.precond == 1)
          out[3 * u + i] = B[i] * in[3 * u] + B[i + 3] * in[3 * u + 1] + B[i + 6] * in[3 * u + 2];
        else
          out[3 * u + i] = B[4 * i] * in[3 * u + i];
      }
    }
  };
  const double rhsNorm2 = dot(rhs, rhs);
  s.lastIters = 0;
  if (rhsNorm2 == 0) {
    s.lastErr = 0;
    return;
  }
  const double threshold = std::max(s.tol * s.tol * rhsNorm2, std::numeric_limits<double>::min());
  double rn2 = dot(r, r);
  if (rn2 < threshold) {
    s.lastErr = std::sqrt(rn2 / rhsNorm2);
    return;
  }
  applyPrec(r, p);
  double absNew = dot(r, p);
  int i = 0;
  while (i < s.maxit) {
    applyLHS(s, A, p, tmp);
    const double alpha = absNew / dot(p, tmp);
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)n; k++) {
      x[k] += alpha * p[k];
      r[k] -= alpha * tmp[k];
    }
    rn2 = dot(r, r);
    if (rn2 < threshold) break;
    applyPrec(r, z);
    const double absOld = absNew;
    absNew = dot(r, z);
    const double beta = absNew / absOld;
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)n; k++) p[k] = z[k] + beta * p[k];
    i++;
  }
  s.lastErr = std::sqrt(rn2 / rhsNorm2);
  s.lastIters = i;
}

// computeCollisionDetection + computeCollisionResponse (TIMESTEPPER.cpp:614-720)
// for a step whose A weighs the collision Hessian H_coll by collScale:
// R += f_coll; the PCG adds collScale H_coll (in pair order) and its
// diagonal blocks to the preconditioner; with collKv, also H_coll v.
// vec: the vector H_coll multiplies for collKv (default: the velocity).
void collisionTerms(Sim& s, double collScale, std::vector<double>* collKv,
                    const std::vector<double>* vec = nullptr) {
  const std::vector<double>& kvOf = vec ? *vec : s.v;
  const int nv = s.M.nv;
  Collisions& C = s.coll;
  C.weight.clear();
  s.collDiag.clear();
  if (!C.on && !C.ee) return;
  if (C.on) {
    vfDetect(s);
    vfResponse(s);
  } else {
    C.pairs.clear();
    C.ctets.clear();
    C.f12.clear();
    C.H12.clear();
  }
  C.eePairs.clear();
  if (C.ee) eeCollisions(s);  // appended after the vertex-face pairs (TIMESTEPPER.cpp:665-690)
  s.collScale = collScale;
  std::vector<double> fc(3 * (size_t)nv, 0.0);
  if (collKv) collKv->assign(3 * (size_t)nv, 0.0);
  s.collDiag.assign(9 * (size_t)nv, 0.0);
  for (size_t k = 0; k < C.weight.size(); k++) {
    const double* H = &C.H12[144 * k];
    for (int a = 0; a < 4; a++) {
      const int u = C.ctets[4 * k + a];
      for (int i = 0; i < 3; i++) fc[3 * u + i] += C.f12[12 * k + 3 * a + i];
      for (int b = 0; b < 4; b++) {
        const int w = C.ctets[4 * k + b];
        for (int i = 0; i < 3; i++)
          for (int j = 0; j < 3; j++) {
            const double h = H[(3 * a + i) + 12 * (3 * b + j)];
            if (collKv) (*collKv)[3 * u + i] += h * kvOf[3 * w + j];
            if (u == w && s.free[u]) s.collDiag[9 * (size_t)u + i + 3 * j] += s.collScale * h;
          }
      }
    }
  }
  for (size_t k = 0; k < fc.size(); k++) s.R[k] = s.R[k] + fc[k];
}

// One BACKWARD_EULER_VELOCITY::solveRayleighDamped step with collisions off
// (BACKWARD_EULER_VELOCITY.cpp:107-235).  The Rayleigh C built at line 118 is
// zeroed by computeCollisionResponse (TIMESTEPPER.cpp:657) before use, so it
// is not formed here; with no plane constraints z = 0 (BEV.cpp:52-81).
void step(Sim& s) {
  const Mesh& M = s.M;
  const int nv = M.nv;
  // applyKinematicConstraints (TIMESTEPPER.cpp:105-122)
  for (size_t k = 0; k < s.pinned.size(); k++)
    for (int i = 0; i < 3; i++) s.x[3 * s.pinned[k] + i] = s.pinTarget[3 * k + i];
  assemble(s);
  const double dt = s.dt;
  // R += f_coll, K += H_coll, C = beta H_coll, so A gains -(dt beta + dt^2) H_coll
  std::vector<double> collKv;
  collisionTerms(s, -(dt * s.coll.beta + dt * dt), &collKv);
  // K v
  std::vector<double> Kv(3 * (size_t)nv);
#pragma omp parallel for schedule(static)
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) {
      double acc = 0;
      for (int k = M.rowptr[u]; k < M.rowptr[u + 1]; k++) {
        const double* blk = &s.K[9 * (size_t)k];
        const int w = M.cols[k];
        for (int c = 0; c < 3; c++) acc += blk[i + 3 * c] * s.v[3 * w + c];
      }
      Kv[3 * u + i] = acc;
    }
  // b = dt (R + dt K v + f); rhs = S b; A = M - dt^2 K (BEV.cpp:157-170)
  std::vector<double> rhs(3 * (size_t)nv);
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) {
      const size_t k = 3 * (size_t)u + i;
      const double kv = collKv.empty() ? Kv[k] : Kv[k] + collKv[k];
      const double b = dt * (s.R[k] + dt * kv + s.fext[k]);
      rhs[k] = s.free[u] ? b : 0.0;
    }
  s.A.resize(s.K.size());
  const double dt2 = dt * dt;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)s.K.size(); k++) s.A[k] = -dt2 * s.K[k];
  for (int u = 0; u < nv; u++) {
    double* D = &s.A[9 * (size_t)M.diag[u]];
    const double m = s.density * M.oneRing[u];
    for (int i = 0; i < 3; i++) D[4 * i] = m + D[4 * i];
  }
  std::vector<double> y;
  pcg(s, s.A, rhs, y);
  // v += y; x += dt v; v = S v (BEV.cpp:191-201)
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) {
      const size_t k = 3 * (size_t)u + i;
      s.v[k] = s.v[k] + y[k];
      s.x[k] = s.x[k] + dt * s.v[k];
      if (!s.free[u]) s.v[k] = 0.0;
    }
}

// One BACKWARD_EULER_POSITION::solveRayleighDamped step without plane
// constraints, so z = 0 (BACKWARD_EULER_POSITION.cpp:138-330), with optional
// vertex-face contact (R += f_coll; collisionC = beta H_coll enters A only,
// BEP.cpp:187-208, so A gains -(beta/dt + 1) H_coll):
//   C   = alpha M + beta K0, K0 = clamped Hessian at zero displacement
//         (buildRayleighDampingMatrix, TIMESTEPPER.cpp:213-236)
//   b   = (M/dt - C) v + R + f_ext                              (BEP.cpp:196)
//   A   = M/dt^2 - C/dt - K                                     (BEP.cpp:207)
//   LHS = S A S + (I - S), rhs = S b; x += y; v = (x - x_old)/dt; v = S v
void stepPosition(Sim& s) {
  const Mesh& M = s.M;
  const int nv = M.nv;
  const double dt = s.dt, invDt = 1.0 / dt;
  const std::vector<double> xOld = s.x;  // _positionOld, before the pins move
  for (size_t k = 0; k < s.pinned.size(); k++)
    for (int i = 0; i < 3; i++) s.x[3 * s.pinned[k] + i] = s.pinTarget[3 * k + i];
  if (s.K0.empty()) {
    const std::vector<double> keep = s.x;
    std::fill(s.x.begin(), s.x.end(), 0.0);
    assemble(s);
    s.K0 = s.K;
    s.x = keep;
  }
  assemble(s);
  collisionTerms(s, -(s.coll.beta * invDt + 1.0), nullptr);
  std::vector<double> rhs(3 * (size_t)nv);
#pragma omp parallel for schedule(static)
  for (int u = 0; u < nv; u++) {
    const double m = s.density * M.oneRing[u];
    for (int i = 0; i < 3; i++) {
      double k0v = 0;
      for (int k = M.rowptr[u]; k < M.rowptr[u + 1]; k++) {
        const double* blk = &s.K0[9 * (size_t)k];
        const int w = M.cols[k];
        for (int c = 0; c < 3; c++) k0v += blk[i + 3 * c] * s.v[3 * w + c];
      }
      const size_t q = 3 * (size_t)u + i;
      const double b = (invDt - s.rayAlpha) * m * s.v[q] - s.rayBeta * k0v + s.R[q] + s.fext[q];
      rhs[q] = s.free[u] ? b : 0.0;
    }
  }
  s.A.resize(s.K.size());
  const double cK0 = s.rayBeta * invDt;
#pragma omp parallel for schedule(static)
  for (long k = 0; k < (long)s.K.size(); k++) s.A[k] = -cK0 * s.K0[k] - s.K[k];
  for (int u = 0; u < nv; u++) {
    double* D = &s.A[9 * (size_t)M.diag[u]];
    const double m = s.density * M.oneRing[u];
    for (int i = 0; i < 3; i++) D[4 * i] = m * (invDt * invDt - s.rayAlpha * invDt) + D[4 * i];
  }
  std::vector<double> y;
  pcg(s, s.A, rhs, y);
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) {
      const size_t k = 3 * (size_t)u + i;
      s.x[k] = s.x[k] + y[k];
      s.v[k] = s.free[u] ? invDt * (s.x[k] - xOld[k]) : 0.0;
    }
}

// One NEWMARK::solveRayleighDamped step (NEWMARK.cpp:183-340), no plane
// constraints (z = 0).  computeCollisionResponse receives the Rayleigh C as
// its damping output and overwrites it (TIMESTEPPER.cpp:645-720): C = 0
// without contact, C = beta H_coll with it.  beta = 1/4, gamma = 1/2
// (NEWMARK.cpp:67-76).  Newton: while step < maxNewton and |rhs|^2 > eps
// (NEWMARK.cpp:212-318), detection and response at the iterate:
//   b = M (a0 (x - x_old) - a2 a_old - a1 v_old)
//       - C (a3 (x - x_old) + a4 v_old + a5 a_old) - R - f_ext
//   A = a0 M - a3 C - K;  LHS = S A S + (I - S), rhs = S b;  x -= y
// with R and K including the collision forces and Hessians.
// then v = a3 (x - x_old) + a4 v_old + a5 a_old,
//      a = a0 (x - x_old) - a1 v_old - a2 a_old, both filtered by S.
void stepNewmark(Sim& s) {
  const Mesh& M = s.M;
  const int nv = M.nv;
  const double dt = s.dt, beta = 0.25, gamma = 0.5;
  const double al[6] = {1.0 / (beta * dt * dt),
                        1.0 / (beta * dt),
                        (1.0 - 2.0 * beta) / (2.0 * beta),
                        gamma / (beta * dt),
                        1.0 - gamma / beta,
                        (1.0 - gamma / (2.0 * beta)) * dt};
  if (s.acc.size() != s.x.size()) s.acc.assign(s.x.size(), 0.0);
  const std::vector<double> xOld = s.x, vOld = s.v, aOld = s.acc;
  for (size_t k = 0; k < s.pinned.size(); k++)
    for (int i = 0; i < 3; i++) s.x[3 * s.pinned[k] + i] = s.pinTarget[3 * k + i];
  double maxR = s.newtonEps * 10;
  int step = 0;
  std::vector<double> rhs(3 * (size_t)nv), y;
  while (step < s.maxNewton && maxR > s.newtonEps) {
    assemble(s);
    if (s.greenMu > 0.0) {
      // NEWMARK::solveEnergyDamped (NEWMARK.cpp:344-480): the iterate's
      // velocity S (a3 (x - x_old) + a4 v_old + a5 a_old), Fdot = V DmInv
      // (TET_MESH::computeFdots, TET_MESH.cpp:660-684), and R gains the
      // GREEN_DAMPING force -vol dF/dx^T mu F (F^T Fdot + Fdot^T F)
      // (GREEN_DAMPING.cpp PK1; TET_MESH.cpp:816-860); its Hessian is passed to
      // computeCollisionResponse, which zeroes it, so A is unchanged
      std::vector<double> vi(3 * (size_t)nv);
      for (int u = 0; u < nv; u++)
        for (int i = 0; i < 3; i++) {
          const size_t q = 3 * (size_t)u + i;
          vi[q] = s.free[u] ? al[3] * (s.x[q] - xOld[q]) + al[4] * vOld[q] + al[5] * aOld[q] : 0.0;
        }
      std::vector<double> fd(12 * (size_t)M.nt);
#pragma omp parallel for schedule(static)
      for (int t = 0; t < M.nt; t++) {
        const int* tv = &M.tets[4 * (size_t)t];
        const double* Dinv = &M.DmInv[9 * (size_t)t];
        double Ds[9], Vs[9], F[9], Fd[9];
        for (int a = 0; a < 3; a++)
          for (int i = 0; i < 3; i++) {
            Ds[i + 3 * a] = (M.rest[3 * tv[a + 1] + i] + s.x[3 * tv[a + 1] + i]) - (M.rest[3 * tv[0] + i] + s.x[3 * tv[0] + i]);
            Vs[i + 3 * a] = vi[3 * tv[a + 1] + i] - vi[3 * tv[0] + i];
          }
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) {
            F[i + 3 * j] = Ds[i] * Dinv[3 * j] + Ds[i + 3] * Dinv[1 + 3 * j] + Ds[i + 6] * Dinv[2 + 3 * j];
            Fd[i + 3 * j] = Vs[i] * Dinv[3 * j] + Vs[i + 3] * Dinv[1 + 3 * j] + Vs[i + 6] * Dinv[2 + 3 * j];
          }
        double G[9], P[9];  // G = F^T Fdot + Fdot^T F, P = mu F G
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) {
            double a = 0.0, b = 0.0;
            for (int k = 0; k < 3; k++) {
              a += F[k + 3 * i] * Fd[k + 3 * j];
              b += Fd[k + 3 * i] * F[k + 3 * j];
            }
            G[i + 3 * j] = a + b;
          }
        for (int j = 0; j < 3; j++)
          for (int i = 0; i < 3; i++) {
            double a = 0.0;
            for (int k = 0; k < 3; k++) a += F[i + 3 * k] * G[k + 3 * j];
            P[i + 3 * j] = s.greenMu * a;
          }
        // force on vertex a+1 = -vol P DmInv^T row a; vertex 0 = minus their sum
        const double vol = M.vol[t];
        double f0[3] = {0.0, 0.0, 0.0};
        for (int a = 0; a < 3; a++)
          for (int i = 0; i < 3; i++) {
            double acc = 0.0;
            for (int j = 0; j < 3; j++) acc += P[i + 3 * j] * Dinv[a + 3 * j];
            fd[12 * (size_t)t + 3 * (a + 1) + i] = -vol * acc;
            f0[i] += vol * acc;
          }
        for (int i = 0; i < 3; i++) fd[12 * (size_t)t + i] = f0[i];
      }
      for (int u = 0; u < nv; u++)
        for (int k = M.vtxptr[u]; k < M.vtxptr[u + 1]; k++) {
          const int t = M.vtxinc[k] / 4, a = M.vtxinc[k] % 4;
          for (int i = 0; i < 3; i++) s.R[3 * u + i] += fd[12 * (size_t)t + 3 * a + i];
        }
    }
    // contact: R += f_coll, K += H_coll, C = beta H_coll (A gains
    // -(a3 beta + 1) H_coll; b gains -C times the Newmark velocity term)
    std::vector<double> collKv;
    if (s.coll.on || s.coll.ee) {
      std::vector<double> vt(3 * (size_t)nv);
      for (size_t q = 0; q < vt.size(); q++) vt[q] = al[3] * (s.x[q] - xOld[q]) + al[4] * vOld[q] + al[5] * aOld[q];
      collisionTerms(s, -(al[3] * s.coll.beta + 1.0), &collKv, &vt);
    } else {
      collisionTerms(s, 0.0, nullptr);
    }
    maxR = 0.0;
    for (int u = 0; u < nv; u++) {
      const double m = s.density * M.oneRing[u];
      for (int i = 0; i < 3; i++) {
        const size_t q = 3 * (size_t)u + i;
        const double t = m * (al[0] * (s.x[q] - xOld[q]) - al[2] * aOld[q] - al[1] * vOld[q]);
        double b = t - s.R[q] - s.fext[q];
        if (!collKv.empty()) b -= s.coll.beta * collKv[q];
        rhs[q] = s.free[u] ? b : 0.0;
        maxR += rhs[q] * rhs[q];
      }
    }
    s.A.resize(s.K.size());
#pragma omp parallel for schedule(static)
    for (long k = 0; k < (long)s.K.size(); k++) s.A[k] = -s.K[k];
    for (int u = 0; u < nv; u++) {
      double* D = &s.A[9 * (size_t)M.diag[u]];
      const double m = s.density * M.oneRing[u];
      for (int i = 0; i < 3; i++) D[4 * i] = al[0] * m + D[4 * i];
    }
    pcg(s, s.A, rhs, y);
    for (size_t k = 0; k < s.x.size(); k++) s.x[k] -= y[k];
    step++;
  }
  s.lastNewton = step;
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) {
      const size_t q = 3 * (size_t)u + i;
      const double dx = s.x[q] - xOld[q];
      const double vn = al[3] * dx + al[4] * vOld[q] + al[5] * aOld[q];
      const double an = al[0] * dx - al[1] * vOld[q] - al[2] * aOld[q];
      s.v[q] = s.free[u] ? vn : 0.0;
      s.acc[q] = s.free[u] ? an : 0.0;
    }
}

}  // namespace

extern "C" {

// Per-tet quantities at displacement `disp`; any output pointer may be null.
// fiber: the anisotropic energies' direction (may be null otherwise); H9u:
// the unclamped 9x9 Hessian (HYPERELASTIC.h:44).
int oracle_elements(int nv, int nt, const double* rest, const int* tets, const double* disp, int material, double mu,
                    double lambda, const double* fiber, double* F, double* Sigma, double* psiOut, double* P,
                    double* H9, double* fe, double* He, double* H9u) {
  if (nv <= 0 || nt <= 0 || !rest || !tets || !disp) return -1;
  Mesh M;
  buildMesh(M, nv, nt, rest, tets);
  const MaterialParams mat = makeMaterial(material, mu, lambda, fiber);
#pragma omp parallel for schedule(static)
  for (int t = 0; t < nt; t++) {
    double f[9], U[9], S[3], V[9], fl[12], H[144];
    elementTerms(M, mat, disp, t, f, U, S, V, fl, H);
    if (F) std::memcpy(F + 9 * (size_t)t, f, sizeof(f));
    if (Sigma) std::memcpy(Sigma + 3 * (size_t)t, S, sizeof(S));
    if (psiOut) psiOut[t] = psi(mat, f);
    if (P) PK1(mat, f, P + 9 * (size_t)t);
    if (H9) clampedHessian(mat, U, S, V, H9 + 81 * (size_t)t);
    if (H9u) eigenHessian(mat, U, S, V, H9u + 81 * (size_t)t, false);
    if (fe) std::memcpy(fe + 12 * (size_t)t, fl, sizeof(fl));
    if (He) std::memcpy(He + 144 * (size_t)t, H, sizeof(H));
  }
  return 0;
}

// Rotation-variant SVD of n matrices (column major).
int oracle_svd(int n, const double* F, double* U, double* S, double* V) {
  for (int k = 0; k < n; k++) svd_rv(F + 9 * (size_t)k, U + 9 * (size_t)k, S + 3 * (size_t)k, V + 9 * (size_t)k);
  return 0;
}

void* oracle_create(int nv, int nt, const double* rest, const int* tets, int material, double mu, double lambda,
                    double density, const double* gravity, double dt) {
  if (nv <= 0 || nt <= 0 || !rest || !tets) return nullptr;
  Sim* s = new Sim;
  buildMesh(s->M, nv, nt, rest, tets);
  s->mat = makeMaterial(material, mu, lambda);
  s->density = density;
  s->dt = dt;
  for (int i = 0; i < 3; i++) s->gravity[i] = gravity ? gravity[i] : 0.0;
  s->x.assign(3 * (size_t)nv, 0.0);
  s->v.assign(3 * (size_t)nv, 0.0);
  s->free.assign(nv, 1);
  // externalForces = oneRingVolume * density * g (TIMESTEPPER.cpp:334-345)
  s->fext.resize(3 * (size_t)nv);
  for (int u = 0; u < nv; u++)
    for (int i = 0; i < 3; i++) s->fext[3 * u + i] = s->M.oneRing[u] * (density * s->gravity[i]);
  return s;
}

void oracle_destroy(void* h) { delete static_cast<Sim*>(h); }

// Fibre direction of an anisotropic material (normalised here, as the
// reference constructors do, ANISOTROPIC_ARAP.cpp:26-29).
int oracle_set_fiber(void* h, const double* a) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || !a || !anisotropic(s->mat.kind)) return -1;
  s->mat = makeMaterial(s->mat.kind, s->mat.mu, s->mat.lambda, a);
  return 0;
}

int oracle_set_state(void* h, const double* x, const double* v) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  const size_t n = 3 * (size_t)s->M.nv;
  if (x) s->x.assign(x, x + n);
  if (v) s->v.assign(v, v + n);
  return 0;
}

int oracle_get_state(void* h, double* x, double* v) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  if (x) std::copy(s->x.begin(), s->x.end(), x);
  if (v) std::copy(s->v.begin(), s->v.end(), v);
  return 0;
}

// Pin vertices at their current world position (attachKinematicConstraints,
// TIMESTEPPER.cpp:380-403): target displacement = (rest + x) - rest.
int oracle_attach_pins(void* h, int n, const int* ids) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  for (int k = 0; k < n; k++) {
    const int u = ids[k];
    if (u < 0 || u >= s->M.nv) return -2;
    s->pinned.push_back(u);
    for (int i = 0; i < 3; i++) {
      const double world = s->M.rest[3 * u + i] + s->x[3 * u + i];
      s->pinTarget.push_back(world - s->M.rest[3 * u + i]);
    }
    s->free[u] = 0;
  }
  return 0;
}

// Move the pins: new target displacements (world - rest) for the pinned
// vertices in attach order, as applyKinematicConstraints recomputes them from
// a moved kinematic shape at the start of each solve (TIMESTEPPER.cpp:105-122).
int oracle_set_pin_targets(void* h, int n, const double* targets) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || n != (int)s->pinned.size()) return -1;
  std::copy(targets, targets + 3 * (size_t)n, s->pinTarget.begin());
  return 0;
}

int oracle_set_solver(void* h, double tol, int maxit, int precond) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  s->tol = tol;
  s->maxit = maxit;
  s->precond = precond;
  return 0;
}

int oracle_set_external_forces(void* h, const double* f) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || !f) return -1;
  s->fext.assign(f, f + 3 * (size_t)s->M.nv);
  return 0;
}

int oracle_step(void* h, int nsteps, int* iters, double* errs) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  for (int k = 0; k < nsteps; k++) {
    if (s->integrator == 1) stepPosition(*s);
    else if (s->integrator == 2) stepNewmark(*s);
    else step(*s);
    if (iters) iters[k] = s->lastIters;
    if (errs) errs[k] = s->lastErr;
  }
  return 0;
}

int oracle_nblocks(void* h) { return static_cast<Sim*>(h)->M.rowptr.back(); }

// Integrator: 0 BACKWARD_EULER_VELOCITY, 1 BACKWARD_EULER_POSITION with
// Rayleigh coefficients alpha, beta, 2 NEWMARK (collisions off for 1 and 2).
// Edge-edge pairs of the last step, as surface edge indices, and the surface
// edges themselves (2 ids each).  Returns the pair count (or the edge count
// with pairs == NULL), -1 on a bad handle.
int oracle_ee_pairs(void* h, int* pairs, int* edges) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  const Collisions& C = s->coll;
  if (!pairs) {
    if (edges) std::copy(C.edges.begin(), C.edges.end(), edges);
    return (int)C.edges.size() / 2;
  }
  std::copy(C.eePairs.begin(), C.eePairs.end(), pairs);
  return (int)C.eePairs.size() / 2;
}

// NEWMARK's energy-damped solve with GREEN_DAMPING(mu) (mu = 0: Rayleigh).
// Only NEWMARK reads the damping: set the integrator first; other integrators
// refuse it (the reference's energy-damped BACKWARD_EULER_VELOCITY solve reads
// a never-computed Fdot).
int oracle_set_green_damping(void* h, double mu) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || !(mu >= 0.0) || s->integrator != 2) return -1;
  s->greenMu = mu;
  return 0;
}

int oracle_set_integrator(void* h, int integrator, double alpha, double beta) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || integrator < 0 || integrator > 2) return -1;

  s->integrator = integrator;
  s->rayAlpha = alpha;
  s->rayBeta = beta;
  s->K0.clear();
  return 0;
}

// Vertex-face self collisions on (eps = collision distance, mu = stiffness,
// beta = damping), like TIMESTEPPER's flags and setCollisionEps.
int oracle_set_collisions(void* h, int vf_on, double eps, double mu, double beta) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  s->coll.on = (vf_on & 1) != 0;
  s->coll.ee = (vf_on & 2) != 0;  // bit 1: edge-edge collisions
  s->coll.eps = eps;
  s->coll.mu = mu;
  s->coll.beta = beta;
  if ((s->coll.on || s->coll.ee) && s->coll.tris.empty()) buildSurface(s->M, s->coll);
  return 0;
}

// Detect at the current state; returns the number of pairs and copies up to
// cap (vertex, triangle) pairs.  surface triangles: 3 ints each when tris != NULL.
int oracle_vf_pairs(void* h, int* pairs, int cap, int* tris) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  if (s->coll.tris.empty()) buildSurface(s->M, s->coll);
  vfDetect(*s);
  const int np = (int)s->coll.pairs.size() / 2;
  for (int k = 0; k < std::min(np, cap); k++) {
    pairs[2 * k] = s->coll.pairs[2 * k];
    pairs[2 * k + 1] = s->coll.pairs[2 * k + 1];
  }
  if (tris) std::copy(s->coll.tris.begin(), s->coll.tris.end(), tris);
  return np;
}

// Collision tets, forces (12) and clamped Hessians (144, column major) of the
// pairs found by the last oracle_vf_pairs call.
int oracle_vf_response(void* h, int* tets, double* f12, double* H12) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  vfResponse(*s);
  const size_t np = s->coll.weight.size();
  if (tets) std::copy(s->coll.ctets.begin(), s->coll.ctets.end(), tets);
  if (f12) std::copy(s->coll.f12.begin(), s->coll.f12.end(), f12);
  if (H12) std::copy(s->coll.H12.begin(), s->coll.H12.end(), H12);
  return (int)np;
}

int oracle_num_surface_triangles(void* h) {
  Sim* s = static_cast<Sim*>(h);
  if (s->coll.tris.empty()) buildSurface(s->M, s->coll);
  return (int)s->coll.tris.size() / 3;
}

// BSR pattern (rowptr V+1, cols nblocks) and, at the current displacement,
// the assembled stiffness K (9 per block, column major) and forces R (3V).
int oracle_assemble(void* h, int* rowptr, int* cols, double* K, double* R) {
  Sim* s = static_cast<Sim*>(h);
  if (!s) return -1;
  if (rowptr) std::copy(s->M.rowptr.begin(), s->M.rowptr.end(), rowptr);
  if (cols) std::copy(s->M.cols.begin(), s->M.cols.end(), cols);
  if (K || R) {
    assemble(*s);
    if (K) std::copy(s->K.begin(), s->K.end(), K);
    if (R) std::copy(s->R.begin(), s->R.end(), R);
  }
  return 0;
}

int oracle_newton_iterations(void* h) { return static_cast<Sim*>(h)->lastNewton; }

// NEWMARK's acceleration state (zero before the first NEWMARK step).
int oracle_get_acceleration(void* h, double* a) {
  Sim* s = static_cast<Sim*>(h);
  if (!s || !a) return -1;
  for (size_t k = 0; k < s->x.size(); k++) a[k] = s->acc.size() == s->x.size() ? s->acc[k] : 0.0;
  return 0;
}

double oracle_energy(void* h) {
  Sim* s = static_cast<Sim*>(h);
  double e = 0;
  for (int t = 0; t < s->M.nt; t++) {
    double F[9], U[9], S[3], V[9];
    elementTerms(s->M, s->mat, s->x.data(), t, F, U, S, V, nullptr, nullptr);
    e += s->M.vol[t] * psi(s->mat, F);
  }
  return e;
}

int oracle_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

// Threads of the OpenMP regions that follow (n <= 0: every host core).
int oracle_set_threads(int n) {
#ifdef _OPENMP
  omp_set_num_threads(n > 0 ? n : omp_get_num_procs());
  return omp_get_max_threads();
#else
  (void)n;
  return 1;
#endif
}

}  // extern "C"
