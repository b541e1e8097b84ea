// Shared device-side layout of a packed batch of scenes.
//
// HBM layout (one contiguous region per array, scenes packed back to back):
//   vertices  [V]  rest, displacement x, velocity v, external force, mass,
//                  free mask (0 = pinned), pin target          (interleaved xyz)
//   tets      [T]  int4 global vertex ids, DmInv (9, column major), rest volume,
//                  scene id
//   blocks    [B]  3x3-block CSR of the system matrix: rowptr [V+1] (global),
//                  cols [B] (global vertex ids), values 9 per block ROW major
//   element   [T]  10 upper-triangle 3x3 blocks of the 12x12 element Hessian
//                  (90 values) + 12 right-hand-side contributions
//   maps           block <- (tet, a, b) contributions (CSR by block, ascending
//                  tet), vertex <- (tet, a) incidences (CSR by vertex)
//   tiles          PCG work units: kTileV consecutive vertices of one scene
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace hobak {

enum MaterialKind : int {
  MAT_SNH = 0, MAT_ARAP = 1, MAT_STVK = 2, MAT_LINEAR = 3, MAT_NHBW = 4, MAT_SNHB = 5,
  // anisotropic energies along a fibre direction (Hyperelastic/Volume/ANISOTROPIC_*.cpp)
  MAT_AARAP = 6, MAT_ASTVK = 7, MAT_AFUNG = 8, MAT_ADIR = 9
};
__host__ __device__ __forceinline__ bool is_anisotropic(int kind) { return kind >= MAT_AARAP && kind <= MAT_ADIR; }

constexpr int kTileV = 128;       // default vertices per PCG tile (one CTA)
constexpr int kMinTileV = 64;     // smallest tile size; tile tables are sized for it
//       // vertices per PCG tile (one CTA)
constexpr int kElemHess = 90;     // 10 upper blocks x 9
constexpr int kElemHessStride = 92;  // per-tet stride: each tet's blocks start on a 16-byte boundary
constexpr int kPartials = 4;      // per-tile partial sums slots
// Timesteppers: BACKWARD_EULER_VELOCITY::solve (unknown: the velocity update)
// and BACKWARD_EULER_POSITION::solveRayleighDamped (unknown: the position
// update), sharing every kernel but the coefficients of rhs, LHS and update.
constexpr int kIntegratorVelocity = 0;
constexpr int kIntegratorPosition = 1;
constexpr int kIntegratorNewmark = 2;  // NEWMARK::solveRayleighDamped: a Newton loop of such solves

// Index of block (a, b), a <= b, in the 10-block upper triangle of a 4x4
// block matrix: (0,0)(0,1)(0,2)(0,3)(1,1)(1,2)(1,3)(2,2)(2,3)(3,3).
__host__ __device__ __forceinline__ int upper_block(int a, int b) {
  return a * 4 - (a * (a - 1)) / 2 + (b - a);
}

struct SceneParams {
  int v0, nv;          // vertex range
  int t0, nt;          // tet range
  int tile0, ntiles;   // PCG tile range
  int kind;            // material
  int active;          // 0: the scene is parked (serving) and every kernel skips it
  int pcgCluster;      // > 0: the inner PCG runs in a cluster of this many CTAs (cluster_pcg.cu)
  int integrator;      // kIntegratorVelocity or kIntegratorPosition
  double mu, lambda, alpha;  // reparameterised material constants
  double dt;
  double rayAlpha, rayBeta;  // Rayleigh damping C = rayAlpha M + rayBeta K0 (position integrator)
  double nm[6];              // Newmark coefficients alpha_0..5 (NEWMARK.cpp:71-76) from dt
  double newtonEps;          // Newmark: Newton stops once |rhs|^2 <= newtonEps ...
  int maxNewton;             // ... or after maxNewton iterations
  double fiber[3];           // anisotropic energies: unit fibre direction
  double greenMu;            // Newmark: GREEN_DAMPING mu of the energy-damped solve (0: none)
};

// Per-scene solver scalars, written by the last CTA of each reduction.
// The inner PCG is the Chronopoulos-Gear form of preconditioned CG (one
// reduction phase per kernel); the outer loop is FP64 iterative refinement
// (mixed precision only).
struct SolveState {
  // outer (FP64) system
  double rhsNorm2;     // |rhs|^2
  double threshold;    // max(tol^2 |rhs|^2, DBL_MIN)
  double rr64;         // |rhs - A y|^2 after the last refinement
  double rScale;       // mixed: the FP32 inner solve runs on r64 / rScale (a power of two near |r64|)
  double tol;
  double innerFloor;   // mixed: tightest relative tolerance of an FP32 inner solve
  int outerDone;       // 1 when the step's linear solve is finished
  int sweep;           // refinement sweeps done
  int maxSweeps;       // 1 (FP64) or 1 + max_refinements (mixed)
  int converged;       // 1 converged, 0 not, -1 non-finite
  int totalIters;      // inner iterations summed over sweeps
  int maxit;
  // inner PCG
  double gamma, gammaOld, delta, alpha, beta, rr, innerThreshold;
  float alphaF, betaF;  // FP32 copies for the mixed inner solve (no per-thread conversion)
  int iters, done;
  unsigned ticketA, ticketB;
  // Newmark's Newton loop: iterations done, finished flag, |rhs|^2 of the last one
  int newtonStep, newtonDone;
  double newtonR;
};

}  // namespace hobak
