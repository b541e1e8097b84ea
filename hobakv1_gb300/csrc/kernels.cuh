// Kernel argument blocks and launch wrappers shared by the .cu files.
#pragma once
#include <cuda_runtime.h>

#include "collision.cuh"
#include "common.cuh"

namespace hobak {

// Vectors and matrix of one inner PCG solve, in arithmetic type T.
template <typename T>
struct PcgVecs {
  T* lhs;   // [B][9] row major
  T* minv;  // [V][9] row major
  T* r;     // residual of the inner solve
  T* u;     // preconditioned residual
  T* p;     // search direction
  T* s;     // A p (updated by recurrence)
  T* w;     // A u
  T* d;     // inner solution (the correction)
};

// Tets per staging block of the element kernel (a CTA of 64 or 128 threads
// stages one or two blocks); at most 4 * kStageTets distinct vertices each,
// so a one-byte corner index suffices.
constexpr int kStageTets = 64;

// Cluster-resident PCG (cluster_pcg.cu): scenes solved by clusters of
// 1, 2, 4, 8 or 16 CTAs of kClusterThreads threads (one vertex per thread).
constexpr int kClusterThreads = 1024;
constexpr int kClusterWarps = kClusterThreads / 32;
constexpr int kClusterClasses = 5;           // cluster sizes 1, 2, 4, 8, 16
constexpr int kClusterSmemMax = 200 * 1024;  // dynamic shared memory per CTA, at most
struct ClusterClass {
  int count;          // scenes of this cluster size
  int vpcMax;         // largest vertices per CTA among them (shared-memory sizing)
  const int* scenes;  // device list of their scene ids
};

// Device pointers of one packed batch.  Plain struct passed by value.
// LHS storage: 32-vertex slices of 3x3 blocks (SELL-32).  The row of vertex
// u (blocks k = rowptr[u] + j, j < rowptr[u + 1] - rowptr[u]) lives in the
// slice of vertices [32 (u / 32), 32 (u / 32) + 32), padded to the slice's
// longest row; entry e (row major) of block j sits at
//   lhs[(sliceRow[u / 32] + j) * 288 + 32 e + u % 32]
// and its column at colS[(sliceRow[u / 32] + j) * 32 + u % 32].  A warp over
// 32 consecutive vertices reads one entry of one slot as one 128-byte line.
constexpr int kSlice = 32;
constexpr int kSlotVals = 9 * kSlice;

// A power of two within a factor of two of sqrt(rr) (1 for 0 or non-finite):
// the mixed-precision inner solve runs on r64 / scale, so its FP32 vectors and
// dot products stay in range for any residual size, and an exact power-of-two
// scale leaves every FP32 rounding as it would be unscaled.
__device__ __forceinline__ double pow2_near_norm(double rr) {
  if (!(rr > 0.0) || !isfinite(rr)) return 1.0;
  int e;
  frexp(rr, &e);
  return ldexp(1.0, e / 2);
}

struct DeviceBatch {
  int nscenes, nv, nt, nblocks, ntiles;
  // launch shapes (hobak_batch_autotune): vertices per PCG tile (64 or 128),
  // element-kernel CTA size (64 or 128), assembly CTA size
  int tileV, elemThreads, asmThreads;
  // PCG loop kernels: compacted list of tiles still iterating and its length
  // (k_compact_tiles)
  int* loopTiles;
  int* nLoopTiles;
  int nTileScenes;  // scenes whose inner PCG runs on the tile path (the rest: clusters)
  const SceneParams* scenes;
  SolveState* solve;
  int* active;  // scenes whose inner PCG is still running
  unsigned long long* bodyRuns;  // PCG loop bodies executed (graph mode), for launch accounting

  // vertices
  const double* rest;
  double* x;
  double* v;
  const double* fext;
  const double* mass;
  const unsigned char* freeMask;
  const double* pinTarget;  // 3 per vertex (only pinned entries used)
  const int* vertexScene;

  // tets
  const int4* tets;
  // element-kernel staging (k_element): per block of kStageTets consecutive
  // tets, its distinct vertices (stageVerts[stagePtr[b] .. stagePtr[b + 1]),
  // ascending) and each tet corner's index in that list
  const int* stagePtr;
  const int* stageVerts;
  const uchar4* stageLocal;
  int stageMax;  // most distinct vertices of any two consecutive staging blocks
  const double* DmInv;
  const double* vol;
  const int* tetScene;

  // block sparsity
  const int* rowptr;
  const int* cols;
  const int* blkRow;
  const int* blkptr;  // block <- contributions
  const int* blksrc;  // tet*16 + a*4 + b
  const int* vtxptr;  // vertex <- incidences
  const int* vtxinc;  // tet*4 + a
  // sliced LHS storage (lhs_slot): first slot row of each 32-vertex slice
  // (nslices + 1 entries), the slice of each slot row, and the column of
  // every slot (padding slots: the vertex itself)
  const int* sliceRow;
  const int* slotSlice;
  const int* colS;
  int nslotRows;
  // cluster-resident PCG: per slot, the owner CTA and local index of its
  // column (k_cluster_gather; scenes on the tile path: unused)
  int* clusterGather;
  // clamped Hessian at zero displacement, CSR block order, 3x3 column major
  // (the position integrator's Rayleigh damping; null when unused)
  const double* K0;
  // Newmark: acceleration, the step's starting x, v, a, and the count of
  // scenes whose Newton loop still runs
  double* acc;
  double* xOld;
  double* vOld;
  double* aOld;
  int* newtonActive;
  unsigned long long* newtonRuns;  // Newton loop bodies executed (graph mode), for launch accounting

  // tiles
  const int* tileScene;
  const int* tileV0;
  const int* tileV1;

  // per-tet element outputs
  double* elemH;   // [T][90] FP64 path
  float* elemHf;   // [T][90] mixed path
  double* elemG;   // [T][12]

  // outer FP64 system
  double* rhs;
  double* y;
  double* r64;
  // inner solves
  PcgVecs<double> v64;  // FP64 path (r = r64, d = y)
  PcgVecs<float> v32;   // mixed path
  double* partial;      // [ntiles][kPartials]
  double* psi;          // [T] energy density scratch
  int anyAniso;          // some scene has an anisotropic energy (k_element_aniso)
  int anyArap, anySvdFree;  // some scene has ARAP / another isotropic energy (mixed element kernels)
  int anyGreen;          // some Newmark scene has GREEN_DAMPING (k_green_damping)
  // vertex-face collisions (collOn = 0: none in this batch)
  int collOn;
  DeviceCollisions coll;
};

// Offset of entry 0 of block j of vertex u's row in the sliced LHS (entry e
// at + kSlice * e), and of its column in colS.
__device__ __forceinline__ size_t lhs_slot(const DeviceBatch& b, int u, int j) {
  return (size_t)(b.sliceRow[u >> 5] + j) * kSlotVals + (u & (kSlice - 1));
}
__device__ __forceinline__ size_t col_slot(const DeviceBatch& b, int u, int j) {
  return (size_t)(b.sliceRow[u >> 5] + j) * kSlice + (u & (kSlice - 1));
}

// Weight of the collision Hessian H_coll in the step's matrix A, with
// K += H_coll and collision damping beta H_coll (TIMESTEPPER.cpp:645-720):
// velocity integrator A = M - dt C - dt^2 K gives -(dt beta + dt^2);
// position integrator A = M/dt^2 - (C + collisionC)/dt - K gives
// -(beta/dt + 1) (BACKWARD_EULER_POSITION.cpp:187-208); NEWMARK
// A = a0 M - a3 C - K gives -(a3 beta + 1) (NEWMARK.cpp:257-262).
__device__ __forceinline__ double collision_lhs_scale(const DeviceBatch& b, int s) {
  const double dt = b.scenes[s].dt, beta = b.coll.scenes[s].beta;
  const int integ = b.scenes[s].integrator;
  return integ == kIntegratorPosition  ? -(beta / dt + 1.0)
         : integ == kIntegratorNewmark ? -(b.scenes[s].nm[3] * beta + 1.0)
                                       : -(dt * beta + dt * dt);
}

void launch_begin_step(const DeviceBatch& b, cudaStream_t s);
// rawForces = 1 stores the element force f itself in elemG instead of dt (f + dt He v)
void launch_element(const DeviceBatch& b, cudaStream_t s, int rawForces = 0);
void launch_element_mixed(const DeviceBatch& b, cudaStream_t s);
// NEWMARK energy-damped solve: adds each damped scene's GREEN_DAMPING element
// forces to elemG (after the element kernel; no-op without damped scenes)
void launch_green_damping(const DeviceBatch& b, cudaStream_t s);
// element-phase kernel launches of a batch: k_element, plus k_element_aniso
// and k_green_damping where the batch needs them
inline int element_launches(const DeviceBatch& b, bool mixed) {
  return (mixed ? (b.anyArap ? 1 : 0) + (b.anySvdFree ? 1 : 0) : 1) + (b.anyAniso ? 1 : 0);
}
// K blocks (column major, un-masked, no mass) and R = sum of element forces, for inspection
void launch_assemble_raw(const DeviceBatch& b, double* K, double* R, cudaStream_t s);
template <typename T>
void launch_assemble(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s);
template <typename T>
void launch_diag_inverse(const DeviceBatch& b, const PcgVecs<T>& v, int precond, cudaStream_t s);
void launch_rhs(const DeviceBatch& b, cudaStream_t s);
void launch_set_active(const DeviceBatch& b, cudaStream_t s);
// Grid sizes of the PCG loop kernels: class 0 launches a CTA per tile of
// the batch, the smaller classes a CTA per tile still iterating at most.
constexpr int kGridClasses = 5;
struct GridClasses {
  int n;                   // classes in use (1..kGridClasses)
  int grid[kGridClasses];  // decreasing; grid[0] = ntiles
};
GridClasses grid_classes(int ntiles);
// Compaction of the tiles still iterating; with a switch handle (graph mode)
// it also selects the smallest grid class that covers them.
void launch_compact_tiles(const DeviceBatch& b, cudaStream_t s, unsigned long long switchHandle = 0,
                          const GridClasses* classes = nullptr);
template <typename T>
void launch_inner_init(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s);
template <typename T>
void launch_spmv(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s, bool pdl = false, int grid = 0);
template <typename T>
void launch_update(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s, bool pdl = false, int grid = 0);
template <typename T>
// One PCG iteration.  The update always overlaps the SpMV's drain; the SpMV
// overlaps the previous update's except right after k_compact_tiles (`first`),
// whose tile list it reads before its dependency wait.
void launch_pcg_iteration(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s, bool first = false,
                          int grid = 0) {
  launch_spmv<T>(b, v, s, !first, grid);
  launch_update<T>(b, v, s, true, grid);
}
void launch_refine(const DeviceBatch& b, cudaStream_t s);  // y += d, then r64 = rhs - A y
void launch_continue(const DeviceBatch& b, unsigned long long handle, cudaStream_t s);void launch_finish_step(const DeviceBatch& b, cudaStream_t s);
// Newmark: save x, v, a and start the Newton loop; after each solve
// x -= y and the per-scene Newton test; the graph loop's condition.
void launch_newton_begin(const DeviceBatch& b, cudaStream_t s);
void launch_newton_update(const DeviceBatch& b, cudaStream_t s);
void launch_newton_continue(const DeviceBatch& b, unsigned long long handle, cudaStream_t s);
// Sets a graph conditional handle (a loop's condition before its node).
void launch_set_condition(unsigned long long handle, unsigned value, cudaStream_t s);
void launch_energy(const DeviceBatch& b, cudaStream_t s);

// element-level entry points (standalone, no batch)
// (F or, when U is given, U/S/V input; fiber: anisotropic energies' direction or null)
void launch_material_eval(int kind, double mu, double lambda, const double* fiber, int n, const double* F,
                          const double* U, const double* S, const double* V, double* psi, double* P, double* H,
                          double* Hu, cudaStream_t s);
void launch_element_eval(int nt, const int4* tets, const double* rest, const double* x, const double* DmInv,
                         const double* vol, int kind, double mu, double lambda, const double* fiber, double* F,
                         double* sigma, double* force, double* hessian, cudaStream_t s);

// Inner PCG of every scene of cluster class k (classes[0..4]: cluster sizes
// 1, 2, 4, 8, 16).  Returns a cudaError_t value (0 on success).
template <typename T>
int launch_cluster_pcg(const DeviceBatch& b, const PcgVecs<T>& v, const ClusterClass* classes, int k,
                       cudaStream_t s);
// Rebuilds the cluster kernels' gather table from the scenes' cluster sizes.
void launch_cluster_gather(const DeviceBatch& b, cudaStream_t s);
// Dynamic shared-memory opt-in of the cluster kernels (once, outside capture).
int configure_cluster_pcg();
// Shared memory a cluster CTA needs: fixed part + per-vertex part.
size_t cluster_vertex_bytes(bool mixed);
size_t cluster_fixed_bytes();

}  // namespace hobak
