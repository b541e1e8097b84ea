// Host side of the C ABI (include/hobak_gpu.h): batch set-up (rest-shape
// precompute, block sparsity, element->block maps, tiles), device memory, the
// step driver and the element-level entry points.
#include <cuda_runtime.h>

#include <algorithm>
#include <array>
#include <cmath>
#include <map>
#include <cstdio>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "../../include/hobak_gpu.h"
#include "element_math.cuh"
#include "kernels.cuh"

using namespace hobak;

namespace {

thread_local std::string g_lastError;

int fail(int code, const std::string& msg) {
  g_lastError = msg;
  return code;
}

}  // namespace

namespace hobak {
int record_error(int code, const std::string& msg) { return fail(code, msg); }
}  // namespace hobak

namespace {

#define CUDA_TRY(expr)                                                                          \
  do {                                                                                          \
    cudaError_t _e = (expr);                                                                    \
    if (_e != cudaSuccess)                                                                      \
      return fail(_e == cudaErrorMemoryAllocation ? HOBAK_ERR_NO_MEMORY : HOBAK_ERR_CUDA,       \
                  std::string(#expr) + ": " + cudaGetErrorString(_e));                          \
  } while (0)

// One device allocation carved into aligned sub-buffers.
struct Arena {
  char* base = nullptr;
  size_t size = 0, used = 0;
  std::vector<std::pair<size_t, size_t>> plan;  // (offset, bytes)
  size_t reserve(size_t bytes) {
    used = (used + 255) & ~size_t(255);
    const size_t off = used;
    used += bytes;
    return off;
  }
};

struct SceneHost {
  int nv, nt;
  int v0, t0, b0, tile0, ntiles;
  hobak_material mat;
  double density, dt;
  double gravity[3];
  std::vector<int> pinned;  // global vertex ids, in the order the scene gave them
};

}  // namespace

struct hobak_batch_t {
  std::vector<SceneHost> scenes;
  hobak_solver_opts opts{};
  int nv = 0, nt = 0, nblocks = 0, ntiles = 0;
  std::vector<double> oneRing;   // per vertex
  std::vector<unsigned char> freeMask;
  std::vector<int> tetsHost;     // global ids
  DeviceBatch d{};
  void* arena = nullptr;
  size_t arenaBytes = 0;
  void* precArena = nullptr;  // buffers of the current precision (alloc_precision)
  double* K0 = nullptr;       // rest-state clamped Hessian (position integrator; rest_hessian)
  size_t precBytes = 0;
  bool precMixed = false;
  cudaStream_t stream = nullptr;
  cudaStream_t captureStream = nullptr;   // fills the bodies of captured while loops
  cudaStream_t captureStream2 = nullptr;  // fills the bodies of the switch nodes inside them
  cudaStream_t captureStreamN = nullptr;  // fills the body of a Newmark step's Newton loop
  long long eagerNewton = 0;              // Newton bodies enqueued eagerly
  cudaGraphExec_t stepGraph[2] = {nullptr, nullptr};  // untimed, timed
  long long eagerChunks = 0;
  long long loopLaunchBase = 0;  // loop-body launches folded in before the last chunk change
  int chunk = 8;                 // PCG iterations per loop body (graph) or per host poll (eager)
  int ntilesCap = 0;             // tile tables are sized for the smallest tile size
  // cluster-resident PCG (cluster_pcg.cu): on/off, the classes of the
  // current precision, and whether any scene is left to the tile path
  bool clusterPcg = false;
  int clusterMax = 16;  // largest cluster (CTAs) a scene may use; larger scenes keep the tile path
  bool clusterDirty = true;
  ClusterClass classes[kClusterClasses] = {};
  int* clusterList = nullptr;  // device, nscenes ids grouped by class
  std::vector<int> hostClusterList;  // host copy of clusterList
  bool clusterOrderStale = false;    // new iteration counts since the classes were last ordered
  std::vector<int> sceneCluster;  // per scene: 0 by the tuning, > 0 a cluster size, -1 the tile path
  bool anyTileScene = true;
  cudaStream_t classStream[kClusterClasses] = {};  // classes run beside the tile path (fork/join)
  cudaEvent_t evFork = nullptr, evJoin[kClusterClasses] = {};
  int lastStatus = HOBAK_OK;
  std::vector<SolveState> lastSolve;
  std::vector<int> hostRowptr, hostCols;
  std::vector<SceneParams> sceneParams;   // host copy (active flags)
  SolveState* solvePinned = nullptr;      // pinned landing buffer for per-step stats
  bool pending = false;                   // steps enqueued, stats not collected yet
  std::vector<double> restHost;  // rest positions (surface areas for collisions)
  std::vector<double> pinTargetHost;  // host copy of the pin targets (3 per vertex)
  // vertex-face collisions
  std::vector<CollisionScene> collScenes;
  std::vector<int> surfTri, surfTriStart, svHost, svStart;  // global ids; per-scene ranges
  std::vector<int> edgeHost, edgeStart;                     // surface edges (lo, hi), global ids; per-scene ranges
  void* collArena = nullptr;
  size_t collBytes = 0;
  int* pinnedActive = nullptr;   // pinned host word for the convergence poll
  long long launches = 0;        // kernels launched by this batch
  bool timing = false;
  cudaEvent_t ev[6] = {};
  double phaseMs[5] = {0, 0, 0, 0, 0};
  long long phaseLaunches[5] = {0, 0, 0, 0, 0};
};

namespace {


double tet_volume(const double* x0, const double* x1, const double* x2, const double* x3) {
  const double d1[3] = {x1[0] - x0[0], x1[1] - x0[1], x1[2] - x0[2]};
  const double d2[3] = {x2[0] - x0[0], x2[1] - x0[1], x2[2] - x0[2]};
  const double d3[3] = {x3[0] - x0[0], x3[1] - x0[1], x3[2] - x0[2]};
  const double c[3] = {d1[1] * d2[2] - d1[2] * d2[1], d1[2] * d2[0] - d1[0] * d2[2], d1[0] * d2[1] - d1[1] * d2[0]};
  return (d3[0] * c[0] + d3[1] * c[1] + d3[2] * c[2]) / 6.0;
}

// DmInv by cofactors (TET_MESH.cpp:178-191 inverts Dm with Eigen).
void dm_inverse(const double* x0, const double* x1, const double* x2, const double* x3, double* Ai) {
  double A[9];
  for (int i = 0; i < 3; i++) {
    A[i] = x1[i] - x0[i];
    A[3 + i] = x2[i] - x0[i];
    A[6 + i] = x3[i] - x0[i];
  }
  const double det = A[0] * (A[4] * A[8] - A[7] * A[5]) - A[3] * (A[1] * A[8] - A[7] * A[2]) +
                     A[6] * (A[1] * A[5] - A[4] * A[2]);
  const double id = 1.0 / det;
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

// A known kind; the anisotropic energies need a non-zero, finite fibre.
int validate_material(const hobak_material& m, int idx) {
  char buf[160];
  if (m.kind < HOBAK_MATERIAL_SNH || m.kind > HOBAK_MATERIAL_ANISOTROPIC_DIRICHLET) {
    std::snprintf(buf, sizeof(buf), "scene %d: unknown material kind %d", idx, m.kind);
    return fail(HOBAK_ERR_INVALID, buf);
  }
  if (is_anisotropic(m.kind)) {
    const double n2 = m.fiber[0] * m.fiber[0] + m.fiber[1] * m.fiber[1] + m.fiber[2] * m.fiber[2];
    if (!(n2 > 0.0) || !std::isfinite(n2)) {
      std::snprintf(buf, sizeof(buf), "scene %d: anisotropic material needs a non-zero fibre direction", idx);
      return fail(HOBAK_ERR_INVALID, buf);
    }
  }
  return HOBAK_OK;
}

int validate_scene(const hobak_scene_desc& s, int idx) {
  char buf[160];
  if (s.nv <= 0 || s.nt <= 0 || !s.rest || !s.tets) {
    std::snprintf(buf, sizeof(buf), "scene %d: empty mesh or null rest/tets", idx);
    return fail(HOBAK_ERR_INVALID, buf);
  }
  if (int rc = validate_material(s.material, idx)) return rc;
  if (!(s.dt > 0.0) || !(s.density > 0.0)) {
    std::snprintf(buf, sizeof(buf), "scene %d: dt and density must be positive", idx);
    return fail(HOBAK_ERR_INVALID, buf);
  }
  if (s.npinned < 0 || (s.npinned > 0 && !s.pinned)) {
    std::snprintf(buf, sizeof(buf), "scene %d: bad pin list", idx);
    return fail(HOBAK_ERR_INVALID, buf);
  }
  for (long k = 0; k < 4L * s.nt; k++)
    if (s.tets[k] < 0 || s.tets[k] >= s.nv) {
      std::snprintf(buf, sizeof(buf), "scene %d: tet vertex id out of range at %ld", idx, k);
      return fail(HOBAK_ERR_INVALID, buf);
    }
  for (int k = 0; k < s.npinned; k++)
    if (s.pinned[k] < 0 || s.pinned[k] >= s.nv) {
      std::snprintf(buf, sizeof(buf), "scene %d: pinned id out of range", idx);
      return fail(HOBAK_ERR_INVALID, buf);
    }
  return HOBAK_OK;
}

template <typename T>
T* carve(void* base, size_t off) {
  return reinterpret_cast<T*>(static_cast<char*>(base) + off);
}

void drop_graphs(hobak_batch_t* B);

// A scene's integrator constants: Rayleigh coefficients (position) and the
// Newmark coefficients for beta = 1/4, gamma = 1/2 from its dt
// (NEWMARK.cpp:67-76, recomputed by setDt at NEWMARK.cpp:107-116).
void set_integrator(SceneParams& p, const hobak_solver_opts& o) {
  p.integrator = o.integrator;
  p.rayAlpha = o.rayleigh_alpha;
  p.rayBeta = o.rayleigh_beta;
  const double dt = p.dt, beta = 0.25, gamma = 0.5;
  p.nm[0] = 1.0 / (beta * dt * dt);
  p.nm[1] = 1.0 / (beta * dt);
  p.nm[2] = (1.0 - 2.0 * beta) / (2.0 * beta);
  p.nm[3] = gamma / (beta * dt);
  p.nm[4] = 1.0 - gamma / beta;
  p.nm[5] = (1.0 - gamma / (2.0 * beta)) * dt;
  p.newtonEps = o.newton_tolerance;
  p.maxNewton = o.max_newton;
}

// Clamped Hessian of every scene at zero displacement (the position
// integrator's Rayleigh damping C = alpha M + beta K0 builds it at rest every
// step, TIMESTEPPER.cpp:213-236; it never changes, so once per batch), FP64,
// CSR block order: element Hessians at x = 0 into scratch, gathered like the
// inspection call's K.  Every scene counts, parked or not.
int rest_hessian(hobak_batch_t* B) {
  if (B->K0) return HOBAK_OK;
  const size_t kBytes = sizeof(double) * 9 * (size_t)std::max(B->nblocks, 1);
  CUDA_TRY(cudaMalloc(&B->K0, kBytes));
  const size_t ehBytes = sizeof(double) * kElemHessStride * (size_t)B->nt, xBytes = sizeof(double) * 3 * (size_t)B->nv;
  void* scratch = nullptr;
  CUDA_TRY(cudaMalloc(&scratch, ehBytes + 2 * xBytes));
  cudaStream_t s = B->stream;
  DeviceBatch d = B->d;
  d.elemH = static_cast<double*>(scratch);
  double* zero = reinterpret_cast<double*>(static_cast<char*>(scratch) + ehBytes);
  double* R = zero + 3 * (size_t)B->nv;
  d.x = zero;
  std::vector<SceneParams> sp = B->sceneParams;
  for (auto& p : sp) p.active = 1;
  cudaError_t e = cudaMemsetAsync(zero, 0, xBytes, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(const_cast<SceneParams*>(d.scenes), sp.data(), sizeof(SceneParams) * sp.size(),
                        cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    launch_element(d, s, 1);
    launch_assemble_raw(d, B->K0, R, s);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(const_cast<SceneParams*>(d.scenes), B->sceneParams.data(),
                        sizeof(SceneParams) * sp.size(), cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(scratch);
  if (e != cudaSuccess) return fail(HOBAK_ERR_CUDA, std::string("rest Hessian: ") + cudaGetErrorString(e));
  B->d.K0 = B->K0;
  drop_graphs(B);
  return HOBAK_OK;
}

// Buffers of the batch's precision, in their own allocation (replaced when
// the precision changes): FP64 element Hessians, sliced LHS, block inverse
// and inner vectors (r = r64, d = y) for the FP64 path, or their FP32
// counterparts for the mixed path.  The other path's pointers are null.
int alloc_precision(hobak_batch_t* B) {
  if (B->precArena) {
    CUDA_TRY(cudaFree(B->precArena));
    B->precArena = nullptr;
    B->precBytes = 0;
  }
  DeviceBatch& d = B->d;
  const size_t nt = (size_t)B->nt, nv = (size_t)B->nv, vals = (size_t)kSlotVals * d.nslotRows;
  const bool mixed = B->opts.precision == HOBAK_PRECISION_MIXED;
  const size_t w = mixed ? sizeof(float) : sizeof(double);
  Arena A;
  const size_t oEH = A.reserve(w * kElemHessStride * nt);
  const size_t oLhs = A.reserve(w * vals);
  const size_t oMinv = A.reserve(w * 9 * nv);
  size_t oVec[6];
  for (int k = 0; k < (mixed ? 6 : 4); k++) oVec[k] = A.reserve(w * 3 * nv);
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, A.used);
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? HOBAK_ERR_NO_MEMORY : HOBAK_ERR_CUDA,
                std::string("cudaMalloc of precision buffers: ") + cudaGetErrorString(e));
  B->precArena = base;
  B->precBytes = A.used;
  CUDA_TRY(cudaMemset(base, 0, A.used));
  if (mixed) {
    d.elemH = nullptr;
    d.elemHf = carve<float>(base, oEH);
    d.v64 = PcgVecs<double>{};
    d.v32 = PcgVecs<float>{carve<float>(base, oLhs), carve<float>(base, oMinv), carve<float>(base, oVec[0]),
                           carve<float>(base, oVec[1]), carve<float>(base, oVec[2]), carve<float>(base, oVec[3]),
                           carve<float>(base, oVec[4]), carve<float>(base, oVec[5])};
  } else {
    d.elemHf = nullptr;
    d.elemH = carve<double>(base, oEH);
    d.v32 = PcgVecs<float>{};
    d.v64 = PcgVecs<double>{carve<double>(base, oLhs), carve<double>(base, oMinv), d.r64,
                            carve<double>(base, oVec[0]), carve<double>(base, oVec[1]), carve<double>(base, oVec[2]),
                            carve<double>(base, oVec[3]), d.y};
  }
  B->precMixed = mixed;
  return HOBAK_OK;
}

int build_batch(hobak_batch_t* B, const hobak_scene_desc* descs, int n) {
  // ---- host precompute ----
  std::vector<int> vtxptr, vtxinc, rowptr, cols, blkRow, blkptr, blksrc, tileScene, tileV0, tileV1;
  std::vector<int> tetScene, vertexScene;
  std::vector<double> rest, x, v, fext, mass, pinTarget, DmInv, vol;
  std::vector<SceneParams> sparams;
  B->scenes.resize(n);
  int nv = 0, nt = 0;
  for (int s = 0; s < n; s++) {
    B->scenes[s].v0 = nv;
    B->scenes[s].t0 = nt;
    nv += descs[s].nv;
    nt += descs[s].nt;
  }
  B->nv = nv;
  B->nt = nt;
  rest.resize(3 * (size_t)nv);
  x.assign(3 * (size_t)nv, 0.0);
  v.assign(3 * (size_t)nv, 0.0);
  fext.resize(3 * (size_t)nv);
  mass.resize(nv);
  pinTarget.assign(3 * (size_t)nv, 0.0);
  B->freeMask.assign(nv, 1);
  B->oneRing.assign(nv, 0.0);
  vertexScene.resize(nv);
  B->tetsHost.resize(4 * (size_t)nt);
  tetScene.resize(nt);
  DmInv.resize(9 * (size_t)nt);
  vol.resize(nt);
  vtxptr.assign(nv + 1, 0);
  rowptr.assign(nv + 1, 0);

  for (int s = 0; s < n; s++) {
    const hobak_scene_desc& D = descs[s];
    SceneHost& H = B->scenes[s];
    H.nv = D.nv;
    H.nt = D.nt;
    H.mat = D.material;
    H.density = D.density;
    H.dt = D.dt;
    for (int i = 0; i < 3; i++) H.gravity[i] = D.gravity[i];
    const int v0 = H.v0, t0 = H.t0;
    std::memcpy(&rest[3 * (size_t)v0], D.rest, 3 * sizeof(double) * D.nv);
    if (D.x0) std::memcpy(&x[3 * (size_t)v0], D.x0, 3 * sizeof(double) * D.nv);
    if (D.v0) std::memcpy(&v[3 * (size_t)v0], D.v0, 3 * sizeof(double) * D.nv);
    for (int u = 0; u < D.nv; u++) vertexScene[v0 + u] = s;
    // per-tet rest data (TET_MESH.cpp:121-191)
    for (int t = 0; t < D.nt; t++) {
      const int* tv = D.tets + 4 * (size_t)t;
      const double* p[4];
      for (int a = 0; a < 4; a++) {
        B->tetsHost[4 * (size_t)(t0 + t) + a] = v0 + tv[a];
        p[a] = D.rest + 3 * (size_t)tv[a];
      }
      vol[t0 + t] = tet_volume(p[0], p[1], p[2], p[3]);
      if (!(vol[t0 + t] > 0.0)) {
        char buf[128];
        std::snprintf(buf, sizeof(buf), "scene %d: tet %d has non-positive rest volume", s, t);
        return fail(HOBAK_ERR_INVALID, buf);
      }
      dm_inverse(p[0], p[1], p[2], p[3], &DmInv[9 * (size_t)(t0 + t)]);
      tetScene[t0 + t] = s;
    }
    // one-ring volumes: quarter of each incident tet, in tet order (TET_MESH.cpp:156-173)
    for (int t = 0; t < D.nt; t++) {
      const double q = 0.25 * vol[t0 + t];
      for (int a = 0; a < 4; a++) B->oneRing[v0 + D.tets[4 * (size_t)t + a]] += q;
    }
    for (int u = 0; u < D.nv; u++) {
      const double orv = B->oneRing[v0 + u];
      mass[v0 + u] = orv * D.density;  // scaleMass(density) (TIMESTEPPER.h:100)
      for (int i = 0; i < 3; i++)  // addGravity(density * g) (TIMESTEPPER.cpp:334-345)
        fext[3 * (size_t)(v0 + u) + i] = orv * (D.density * D.gravity[i]);
    }
    // pins keep the displacement they have when attached: (rest + x) - rest
    for (int k = 0; k < D.npinned; k++) {
      const int u = v0 + D.pinned[k];
      B->scenes[s].pinned.push_back(u);
      B->freeMask[u] = 0;
      for (int i = 0; i < 3; i++) {
        const double world = rest[3 * (size_t)u + i] + x[3 * (size_t)u + i];
        pinTarget[3 * (size_t)u + i] = world - rest[3 * (size_t)u + i];
      }
    }
  }
  // vertex -> (tet, a) incidences, ascending tet
  for (long k = 0; k < 4L * nt; k++) vtxptr[B->tetsHost[k] + 1]++;
  for (int u = 0; u < nv; u++) vtxptr[u + 1] += vtxptr[u];
  vtxinc.resize(4 * (size_t)nt);
  {
    std::vector<int> fill(vtxptr.begin(), vtxptr.end() - 1);
    for (int t = 0; t < nt; t++)
      for (int a = 0; a < 4; a++) vtxinc[fill[B->tetsHost[4 * (size_t)t + a]]++] = 4 * t + a;
  }
  // block rows: sorted unique neighbours through shared tets
  {
    std::vector<int> nb;
    for (int u = 0; u < nv; u++) {
      nb.clear();
      for (int k = vtxptr[u]; k < vtxptr[u + 1]; k++) {
        const int t = vtxinc[k] >> 2;
        for (int a = 0; a < 4; a++) nb.push_back(B->tetsHost[4 * (size_t)t + a]);
      }
      std::sort(nb.begin(), nb.end());
      nb.erase(std::unique(nb.begin(), nb.end()), nb.end());
      rowptr[u + 1] = rowptr[u] + (int)nb.size();
      cols.insert(cols.end(), nb.begin(), nb.end());
    }
  }
  const int nblocks = rowptr[nv];
  B->nblocks = nblocks;
  // sliced LHS storage: 32-vertex slices, each as many slot rows as its
  // longest block row (lhs_slot)
  const int nslices = (nv + kSlice - 1) / kSlice;
  std::vector<int> sliceRow(nslices + 1, 0), slotSlice, colS;
  for (int sl = 0; sl < nslices; sl++) {
    int len = 0;
    for (int u = kSlice * sl; u < std::min(nv, kSlice * (sl + 1)); u++) len = std::max(len, rowptr[u + 1] - rowptr[u]);
    sliceRow[sl + 1] = sliceRow[sl] + len;
  }
  const int nslotRows = sliceRow[nslices];
  slotSlice.resize(nslotRows);
  for (int sl = 0; sl < nslices; sl++)
    for (int r = sliceRow[sl]; r < sliceRow[sl + 1]; r++) slotSlice[r] = sl;
  colS.resize((size_t)nslotRows * kSlice);
  for (int u = 0; u < nv; u++) {
    const int r0 = sliceRow[u / kSlice], lane = u % kSlice;
    for (int r = r0; r < sliceRow[u / kSlice + 1]; r++) {
      const int j = r - r0;
      colS[(size_t)r * kSlice + lane] = j < rowptr[u + 1] - rowptr[u] ? cols[rowptr[u] + j] : u;
    }
  }
  for (int u = nv; u < nslices * kSlice; u++)  // lanes past the last vertex
    for (int r = sliceRow[u / kSlice]; r < sliceRow[u / kSlice + 1]; r++) colS[(size_t)r * kSlice + u % kSlice] = 0;
  blkRow.resize(nblocks);
  for (int u = 0; u < nv; u++)
    for (int k = rowptr[u]; k < rowptr[u + 1]; k++) blkRow[k] = u;
  // block <- (tet, a, b) contributions in ascending tet order
  {
    std::vector<int> where(16 * (size_t)nt);
    blkptr.assign(nblocks + 1, 0);
    for (int t = 0; t < nt; t++)
      for (int a = 0; a < 4; a++)
        for (int bb = 0; bb < 4; bb++) {
          const int u = B->tetsHost[4 * (size_t)t + a], w = B->tetsHost[4 * (size_t)t + bb];
          const int* beg = cols.data() + rowptr[u];
          const int* end = cols.data() + rowptr[u + 1];
          const int k = rowptr[u] + int(std::lower_bound(beg, end, w) - beg);
          where[16 * (size_t)t + 4 * a + bb] = k;
          blkptr[k + 1]++;
        }
    for (int k = 0; k < nblocks; k++) blkptr[k + 1] += blkptr[k];
    blksrc.resize(16 * (size_t)nt);
    std::vector<int> fill(blkptr.begin(), blkptr.end() - 1);
    for (int t = 0; t < nt; t++)
      for (int e = 0; e < 16; e++) blksrc[fill[where[16 * (size_t)t + e]]++] = 16 * t + e;
  }
  // element-kernel staging: per block of kStageTets consecutive tets, its
  // distinct vertices (ascending) and each tet corner's index among them
  const int nsb = (nt + kStageTets - 1) / kStageTets;
  std::vector<int> stagePtr(nsb + 1, 0), stageVerts;
  std::vector<unsigned char> stageLocal(4 * (size_t)nt);
  {
    std::vector<int> ids;
    for (int sb = 0; sb < nsb; sb++) {
      const int t0 = sb * kStageTets, t1 = std::min(nt, t0 + kStageTets);
      ids.assign(B->tetsHost.begin() + 4 * (size_t)t0, B->tetsHost.begin() + 4 * (size_t)t1);
      std::sort(ids.begin(), ids.end());
      ids.erase(std::unique(ids.begin(), ids.end()), ids.end());
      for (int k = 4 * t0; k < 4 * t1; k++)
        stageLocal[k] = (unsigned char)(std::lower_bound(ids.begin(), ids.end(), B->tetsHost[k]) - ids.begin());
      stageVerts.insert(stageVerts.end(), ids.begin(), ids.end());
      stagePtr[sb + 1] = (int)stageVerts.size();
    }
  }
  // tiles: kTileV consecutive vertices of one scene (apply_tile_size changes
  // the size later; the tables are sized for kMinTileV)
  int ntilesCap = 0;
  int anyAniso = 0, anyArap = 0, anySvdFree = 0;
  for (int s = 0; s < n; s++) {
    SceneHost& H = B->scenes[s];
    ntilesCap += (H.nv + kMinTileV - 1) / kMinTileV;
    H.tile0 = (int)tileScene.size();
    for (int u = 0; u < H.nv; u += kTileV) {
      tileScene.push_back(s);
      tileV0.push_back(H.v0 + u);
      tileV1.push_back(H.v0 + std::min(H.nv, u + kTileV));
    }
    H.ntiles = (int)tileScene.size() - H.tile0;
    H.b0 = rowptr[H.v0];
    const MatParams mp = make_material(H.mat.kind, H.mat.mu, H.mat.lambda, H.mat.fiber);
    SceneParams p{};
    p.v0 = H.v0;
    p.nv = H.nv;
    p.t0 = H.t0;
    p.nt = H.nt;
    p.tile0 = H.tile0;
    p.ntiles = H.ntiles;
    p.kind = mp.kind;
    p.mu = mp.mu;
    p.lambda = mp.lambda;
    p.alpha = mp.alpha;
    for (int i = 0; i < 3; i++) p.fiber[i] = mp.a[i];
    if (is_anisotropic(mp.kind)) anyAniso = 1;
    else if (mp.kind == MAT_ARAP) anyArap = 1;
    else anySvdFree = 1;
    p.dt = H.dt;
    set_integrator(p, B->opts);
    p.active = 1;
    sparams.push_back(p);
  }
  const int ntiles = (int)tileScene.size();
  B->ntiles = ntiles;
  B->ntilesCap = ntilesCap;

  // ---- device arena ----
  Arena A;
  const size_t V3 = 3 * (size_t)nv * sizeof(double);
  struct Slot {
    size_t off;
  };
  const size_t oScenes = A.reserve(sizeof(SceneParams) * n);
  const size_t oSolve = A.reserve(sizeof(SolveState) * n);
  const size_t oActive = A.reserve(sizeof(int));
  const size_t oBodyRuns = A.reserve(sizeof(unsigned long long));
  const size_t oRest = A.reserve(V3), oX = A.reserve(V3), oV = A.reserve(V3), oF = A.reserve(V3);
  const size_t oMass = A.reserve(sizeof(double) * nv), oFree = A.reserve(nv), oPin = A.reserve(V3);
  const size_t oVS = A.reserve(sizeof(int) * nv);
  const size_t oTets = A.reserve(sizeof(int4) * nt), oDm = A.reserve(sizeof(double) * 9 * (size_t)nt);
  const size_t oStagePtr = A.reserve(sizeof(int) * (nsb + 1)), oStageVerts = A.reserve(sizeof(int) * stageVerts.size());
  const size_t oStageLocal = A.reserve(4 * (size_t)nt);
  const size_t oVol = A.reserve(sizeof(double) * nt), oTS = A.reserve(sizeof(int) * nt);
  const size_t oRowptr = A.reserve(sizeof(int) * (nv + 1)), oCols = A.reserve(sizeof(int) * nblocks);
  const size_t oBlkRow = A.reserve(sizeof(int) * nblocks), oBlkptr = A.reserve(sizeof(int) * (nblocks + 1));
  const size_t oBlksrc = A.reserve(sizeof(int) * 16 * (size_t)nt);
  const size_t oVtxptr = A.reserve(sizeof(int) * (nv + 1)), oVtxinc = A.reserve(sizeof(int) * 4 * (size_t)nt);
  const size_t oSliceRow = A.reserve(sizeof(int) * (nslices + 1)), oSlotSlice = A.reserve(sizeof(int) * nslotRows);
  const size_t oColS = A.reserve(sizeof(int) * kSlice * (size_t)nslotRows);
  const size_t oGather = A.reserve(sizeof(int) * kSlice * (size_t)nslotRows);

  const size_t oTileS = A.reserve(sizeof(int) * ntilesCap), oTile0 = A.reserve(sizeof(int) * ntilesCap);
  const size_t oTile1 = A.reserve(sizeof(int) * ntilesCap);
  const size_t oLoopTiles = A.reserve(sizeof(int) * ntilesCap), oNLoop = A.reserve(sizeof(int));
  const size_t oClusterList = A.reserve(sizeof(int) * n);
  const size_t oEG = A.reserve(sizeof(double) * 12 * (size_t)nt);
  const size_t oRhs = A.reserve(V3), oY = A.reserve(V3), oR64 = A.reserve(V3);
  // Newmark: acceleration and the step's starting x, v, a
  const size_t oAcc = A.reserve(V3), oXo = A.reserve(V3), oVo = A.reserve(V3), oAo = A.reserve(V3);
  const size_t oNewton = A.reserve(sizeof(int)), oNewtonRuns = A.reserve(sizeof(unsigned long long));
  const size_t oPart = A.reserve(sizeof(double) * kPartials * (size_t)ntilesCap);
  const size_t oPsi = A.reserve(sizeof(double) * nt);
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, A.used);
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? HOBAK_ERR_NO_MEMORY : HOBAK_ERR_CUDA,
                std::string("cudaMalloc of batch arena: ") + cudaGetErrorString(e));
  B->arena = base;
  B->arenaBytes = A.used;
  CUDA_TRY(cudaMemset(base, 0, A.used));

  DeviceBatch& d = B->d;
  d.nscenes = n;
  d.nv = nv;
  d.nt = nt;
  d.nblocks = nblocks;
  d.ntiles = ntiles;
  d.tileV = kTileV;
  d.elemThreads = 128;
  d.asmThreads = 64;  // the fastest measured on the 7.2 M-tet mix (1.48 ms; 256 threads: 1.70)
  d.scenes = carve<SceneParams>(base, oScenes);
  d.solve = carve<SolveState>(base, oSolve);
  d.active = carve<int>(base, oActive);
  d.bodyRuns = carve<unsigned long long>(base, oBodyRuns);
  d.acc = carve<double>(base, oAcc);
  d.xOld = carve<double>(base, oXo);
  d.vOld = carve<double>(base, oVo);
  d.aOld = carve<double>(base, oAo);
  d.newtonActive = carve<int>(base, oNewton);
  d.newtonRuns = carve<unsigned long long>(base, oNewtonRuns);
  d.rest = carve<double>(base, oRest);
  d.x = carve<double>(base, oX);
  d.v = carve<double>(base, oV);
  d.fext = carve<double>(base, oF);
  d.mass = carve<double>(base, oMass);
  d.freeMask = carve<unsigned char>(base, oFree);
  d.pinTarget = carve<double>(base, oPin);
  d.vertexScene = carve<int>(base, oVS);
  d.tets = carve<int4>(base, oTets);
  d.stagePtr = carve<int>(base, oStagePtr);
  d.stageVerts = carve<int>(base, oStageVerts);
  d.stageLocal = carve<uchar4>(base, oStageLocal);
  d.stageMax = 1;
  for (int sb = 0; sb < nsb; sb += 1)  // a 128-tet CTA stages blocks 2k and 2k + 1
    d.stageMax = std::max(d.stageMax, stagePtr[std::min(nsb, sb + 2)] - stagePtr[sb]);
  d.DmInv = carve<double>(base, oDm);
  d.vol = carve<double>(base, oVol);
  d.tetScene = carve<int>(base, oTS);
  d.rowptr = carve<int>(base, oRowptr);
  d.cols = carve<int>(base, oCols);
  d.blkRow = carve<int>(base, oBlkRow);
  d.blkptr = carve<int>(base, oBlkptr);
  d.blksrc = carve<int>(base, oBlksrc);
  d.vtxptr = carve<int>(base, oVtxptr);
  d.vtxinc = carve<int>(base, oVtxinc);
  d.sliceRow = carve<int>(base, oSliceRow);
  d.slotSlice = carve<int>(base, oSlotSlice);
  d.colS = carve<int>(base, oColS);
  d.clusterGather = carve<int>(base, oGather);
  d.nslotRows = nslotRows;
  d.tileScene = carve<int>(base, oTileS);
  d.tileV0 = carve<int>(base, oTile0);
  d.tileV1 = carve<int>(base, oTile1);
  d.loopTiles = carve<int>(base, oLoopTiles);
  d.nTileScenes = n;
  B->clusterList = carve<int>(base, oClusterList);
  d.nLoopTiles = carve<int>(base, oNLoop);
  d.elemG = carve<double>(base, oEG);
  d.rhs = carve<double>(base, oRhs);
  d.y = carve<double>(base, oY);
  d.r64 = carve<double>(base, oR64);
  d.partial = carve<double>(base, oPart);
  d.psi = carve<double>(base, oPsi);
  d.anyAniso = anyAniso;
  d.anyArap = anyArap;
  d.anySvdFree = anySvdFree;

  auto up = [&](const void* dst, const void* src, size_t bytes) {
    return cudaMemcpy(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice);
  };
  CUDA_TRY(up(d.scenes, sparams.data(), sizeof(SceneParams) * n));
  B->sceneParams = sparams;
  CUDA_TRY(up(d.rest, rest.data(), V3));
  CUDA_TRY(up(d.x, x.data(), V3));
  CUDA_TRY(up(d.v, v.data(), V3));
  CUDA_TRY(up(d.fext, fext.data(), V3));
  CUDA_TRY(up(d.mass, mass.data(), sizeof(double) * nv));
  CUDA_TRY(up(d.freeMask, B->freeMask.data(), nv));
  CUDA_TRY(up(d.pinTarget, pinTarget.data(), V3));
  B->pinTargetHost = pinTarget;
  CUDA_TRY(up(d.vertexScene, vertexScene.data(), sizeof(int) * nv));
  CUDA_TRY(up(d.tets, B->tetsHost.data(), sizeof(int4) * nt));
  CUDA_TRY(up(d.stagePtr, stagePtr.data(), sizeof(int) * (nsb + 1)));
  CUDA_TRY(up(d.stageVerts, stageVerts.data(), sizeof(int) * stageVerts.size()));
  CUDA_TRY(up(d.stageLocal, stageLocal.data(), 4 * (size_t)nt));
  CUDA_TRY(up(d.DmInv, DmInv.data(), sizeof(double) * 9 * (size_t)nt));
  CUDA_TRY(up(d.vol, vol.data(), sizeof(double) * nt));
  CUDA_TRY(up(d.tetScene, tetScene.data(), sizeof(int) * nt));
  CUDA_TRY(up(d.rowptr, rowptr.data(), sizeof(int) * (nv + 1)));
  CUDA_TRY(up(d.cols, cols.data(), sizeof(int) * nblocks));
  CUDA_TRY(up(d.blkRow, blkRow.data(), sizeof(int) * nblocks));
  CUDA_TRY(up(d.blkptr, blkptr.data(), sizeof(int) * (nblocks + 1)));
  CUDA_TRY(up(d.blksrc, blksrc.data(), sizeof(int) * 16 * (size_t)nt));
  CUDA_TRY(up(d.vtxptr, vtxptr.data(), sizeof(int) * (nv + 1)));
  CUDA_TRY(up(d.vtxinc, vtxinc.data(), sizeof(int) * 4 * (size_t)nt));
  CUDA_TRY(up(d.sliceRow, sliceRow.data(), sizeof(int) * (nslices + 1)));
  CUDA_TRY(up(d.slotSlice, slotSlice.data(), sizeof(int) * nslotRows));
  CUDA_TRY(up(d.colS, colS.data(), sizeof(int) * kSlice * (size_t)nslotRows));
  CUDA_TRY(up(d.tileScene, tileScene.data(), sizeof(int) * ntiles));
  CUDA_TRY(up(d.tileV0, tileV0.data(), sizeof(int) * ntiles));
  CUDA_TRY(up(d.tileV1, tileV1.data(), sizeof(int) * ntiles));
  B->hostRowptr = rowptr;
  B->restHost = rest;
  B->hostCols = cols;
  return alloc_precision(B);
}

int sweeps_of(const hobak_solver_opts& o);

int upload_solver_opts(hobak_batch_t* B) {
  std::vector<SolveState> st(B->scenes.size());
  for (auto& s : st) {
    std::memset(&s, 0, sizeof(s));
    s.tol = B->opts.tol;
    s.innerFloor = B->opts.inner_tolerance;
    s.maxit = B->opts.max_iters;
    s.maxSweeps = sweeps_of(B->opts);
  }
  CUDA_TRY(cudaMemcpy(B->d.solve, st.data(), sizeof(SolveState) * st.size(), cudaMemcpyHostToDevice));
  return HOBAK_OK;
}

int check_opts(const hobak_solver_opts* o) {
  if (!o) return HOBAK_OK;
  if (!(o->tol > 0.0) || o->max_iters <= 0) return fail(HOBAK_ERR_INVALID, "solver tol and max_iters must be > 0");
  if (o->precision != HOBAK_PRECISION_FP64 && o->precision != HOBAK_PRECISION_MIXED)
    return fail(HOBAK_ERR_INVALID, "unknown precision mode");
  if (o->preconditioner != HOBAK_PRECOND_JACOBI && o->preconditioner != HOBAK_PRECOND_BLOCK_JACOBI)
    return fail(HOBAK_ERR_INVALID, "unknown preconditioner");
  if (o->max_refinements < 0 || o->max_refinements > 3) return fail(HOBAK_ERR_INVALID, "max_refinements in 0..3");
  if (o->integrator != HOBAK_INTEGRATOR_VELOCITY && o->integrator != HOBAK_INTEGRATOR_POSITION &&
      o->integrator != HOBAK_INTEGRATOR_NEWMARK)
    return fail(HOBAK_ERR_INVALID, "unknown integrator");
  if (o->max_newton < 1 || o->max_newton > 100 || !(o->newton_tolerance >= 0.0))
    return fail(HOBAK_ERR_INVALID, "max_newton in 1..100 and newton_tolerance >= 0");
  if (!(o->inner_tolerance >= 1e-7 && o->inner_tolerance < 1.0))
    return fail(HOBAK_ERR_INVALID, "inner_tolerance in [1e-7, 1)");
  if (!(o->rayleigh_alpha >= 0.0) || !(o->rayleigh_beta >= 0.0) || !std::isfinite(o->rayleigh_alpha) ||
      !std::isfinite(o->rayleigh_beta))
    return fail(HOBAK_ERR_INVALID, "Rayleigh coefficients must be finite and >= 0");
  return HOBAK_OK;
}

int sweeps_of(const hobak_solver_opts& o) {
  return o.precision == HOBAK_PRECISION_MIXED ? 1 + o.max_refinements : 1;
}

// Kernels launched per step outside the PCG loop bodies.
// Kernels of one linear solve outside the PCG loop bodies.
long long solve_launches(const hobak_batch_t* B) {
  const int sweeps = sweeps_of(B->opts);
  const bool mixed = B->opts.precision == HOBAK_PRECISION_MIXED;
  int cl = 0;
  for (const ClusterClass& c : B->classes) cl += c.count > 0 ? 1 : 0;
  // the cluster classes once; per sweep of the tile path: k_set_active,
  // inner init (+ the loop's arming kernel in a graph), the refinement
  if (!B->anyTileScene) return cl;
  return cl + sweeps * (2 + (B->opts.use_graph ? 1 : 0) + (mixed ? 2 : 0));
}

// Kernels of one Newton loop body (Newmark) outside the PCG loop bodies and
// k_newton_continue: element, assembly, preconditioner, rhs, the solve, and
// the update + test.
long long newton_body_launches(const hobak_batch_t* B) {
  return 3 + element_launches(B->d, B->opts.precision == HOBAK_PRECISION_MIXED) + (B->d.anyGreen ? 1 : 0) +
         (B->d.collOn ? collision_launches(B->d.coll) : 0) + solve_launches(B) + 2;
}

long long fixed_launches(const hobak_batch_t* B) {
  // begin, Newton begin, finish (+ the Newton loop's arming kernel in a graph)
  if (B->opts.integrator == HOBAK_INTEGRATOR_NEWMARK) return 3 + (B->opts.use_graph ? 1 : 0);
  return 5 + element_launches(B->d, B->opts.precision == HOBAK_PRECISION_MIXED) +
         (B->d.collOn ? collision_launches(B->d.coll) : 0) + solve_launches(B);
}

void drop_graphs(hobak_batch_t* B);

// Longest first: within each class, the scenes that iterated most in the
// last step (then the larger ones) come first, so that their clusters start
// at the head of the launch and the short solves fill the SMs around them.
// A scene's solve does not depend on where it sits in the list.
void order_cluster_classes(const hobak_batch_t* B, std::vector<int>& list) {
  const bool known = B->lastSolve.size() == B->scenes.size();
  auto key = [&](int s) { return known ? B->lastSolve[s].totalIters : 0; };
  size_t at = 0;
  for (int k = 0; k < kClusterClasses; k++) {
    const size_t end = at + B->classes[k].count;
    std::stable_sort(list.begin() + at, list.begin() + end, [&](int a, int b) {
      const int ka = key(a), kb = key(b);
      if (ka != kb) return ka > kb;
      return B->scenes[a].nv > B->scenes[b].nv;
    });
    at = end;
  }
}

// Re-orders the classes after a step whose iteration counts were collected;
// the graphs read the list at run time, so they stay valid.
int reorder_cluster_classes(hobak_batch_t* B) {
  if (!B->clusterOrderStale || B->hostClusterList.empty()) return HOBAK_OK;
  B->clusterOrderStale = false;
  std::vector<int> list = B->hostClusterList;
  order_cluster_classes(B, list);
  if (list == B->hostClusterList) return HOBAK_OK;
  B->hostClusterList = list;
  // from pageable memory: the call returns once the list is staged
  CUDA_TRY(cudaMemcpyAsync(B->clusterList, B->hostClusterList.data(), sizeof(int) * list.size(),
                           cudaMemcpyHostToDevice, B->stream));
  return HOBAK_OK;
}

// Which scenes solve their inner PCG in a thread-block cluster, and in how
// large a one, for the current precision (a scene in contact adds its
// contact rows in the cluster as the tile path does): the
// smallest cluster (1, 2, 4, 8 or 16 CTAs, at most clusterMax) that gives
// each thread at most one vertex, or else the largest allowed cluster, whose
// threads then take several vertices, as long as its vectors fit in shared
// memory (fewer SMs per scene, more scenes at once; for a scene of up to ~40 k
// vertices in mixed precision, one 16-CTA cluster beats the tile path's two
// grid-wide kernels per iteration); larger scenes keep the tile path, which
// spreads them wider.  The choice depends only on the scene itself, so
// a scene takes the same path alone and in any batch.  Runs outside graph
// capture (it uploads); drops the graphs when the assignment changed.
int prepare_cluster_classes(hobak_batch_t* B) {
  if (!B->clusterDirty) return HOBAK_OK;
  if (const int ce = configure_cluster_pcg())
    return fail(HOBAK_ERR_CUDA, std::string("cluster PCG set-up: ") + cudaGetErrorString((cudaError_t)ce));
  const int n = (int)B->scenes.size();
  const bool mixed = B->opts.precision == HOBAK_PRECISION_MIXED;
  const int vpcLimit = (int)((kClusterSmemMax - cluster_fixed_bytes()) / cluster_vertex_bytes(mixed));
  std::vector<int> cl(n, 0);
  for (int s = 0; s < n; s++) {
    if (!B->clusterPcg) continue;
    const int nv = B->scenes[s].nv;
    const int force = s < (int)B->sceneCluster.size() ? B->sceneCluster[s] : 0;
    if (force < 0) continue;  // this scene keeps the tile path
    if (force > 0) {  // this scene's own cluster size, where its vectors fit
      const int vpcF = (nv + force - 1) / force;
      if (vpcF <= vpcLimit) cl[s] = force;
      continue;
    }
    // the smallest cluster that gives each thread one vertex at most; else
    // the cap, whose threads take several vertices as long as the CTA's
    // vectors fit in its shared memory
    int c = 1;
    while (c < B->clusterMax && (nv + c - 1) / c > kClusterThreads) c *= 2;
    const int vpc = (nv + c - 1) / c;
    if (vpc <= vpcLimit) cl[s] = c;
  }
  std::vector<int> list;
  bool changed = false;
  int nTile = 0;
  const int sizes[kClusterClasses] = {1, 2, 4, 8, 16};
  for (int k = 0; k < kClusterClasses; k++) {
    ClusterClass& c = B->classes[k];
    c.count = 0;
    c.vpcMax = 0;
    c.scenes = B->clusterList + list.size();
    for (int s = 0; s < n; s++)
      if (cl[s] == sizes[k]) {
        list.push_back(s);
        c.count++;
        c.vpcMax = std::max(c.vpcMax, (B->scenes[s].nv + sizes[k] - 1) / sizes[k]);
      }
  }
  order_cluster_classes(B, list);
  B->hostClusterList = list;
  B->clusterOrderStale = false;
  for (int s = 0; s < n; s++) {
    if (B->sceneParams[s].pcgCluster != cl[s]) changed = true;
    B->sceneParams[s].pcgCluster = cl[s];
    if (cl[s] == 0) nTile++;
  }
  B->anyTileScene = nTile > 0;
  if (B->d.nTileScenes != nTile) changed = true;
  B->d.nTileScenes = nTile;
  CUDA_TRY(cudaStreamSynchronize(B->stream));
  if (!list.empty())
    CUDA_TRY(cudaMemcpy(B->clusterList, list.data(), sizeof(int) * list.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(B->d.scenes), B->sceneParams.data(), sizeof(SceneParams) * n,
                      cudaMemcpyHostToDevice));
  if (!list.empty()) {
    launch_cluster_gather(B->d, B->stream);
    CUDA_TRY(cudaGetLastError());
    CUDA_TRY(cudaStreamSynchronize(B->stream));
  }
  if (changed) drop_graphs(B);
  B->clusterDirty = false;
  return HOBAK_OK;
}

// `chunk` PCG iterations (2 kernels each) on `grid` CTAs.
template <typename T>
void enqueue_chunk(const DeviceBatch& d, const PcgVecs<T>& v, cudaStream_t s, int chunk, int grid) {
  for (int c = 0; c < chunk; c++) launch_pcg_iteration<T>(d, v, s, c == 0, grid);
}

// Adds a conditional node of `type` with `size` bodies after the current
// capture dependencies of `s` (which then depend on the node); returns the
// handle and the body graphs.
int add_conditional(cudaStream_t s, cudaGraphConditionalNodeType type, unsigned size, unsigned defaultValue,
                    unsigned flags, cudaGraphConditionalHandle* h, cudaGraph_t* bodies) {
  cudaStreamCaptureStatus cs;
  cudaGraph_t capG = nullptr;
  const cudaGraphNode_t* deps = nullptr;
  size_t nd = 0;
  CUDA_TRY(cudaStreamGetCaptureInfo(s, &cs, nullptr, &capG, &deps, nullptr, &nd));
  if (cs != cudaStreamCaptureStatusActive) return fail(HOBAK_ERR_CUDA, "stream is not capturing");
  CUDA_TRY(cudaGraphConditionalHandleCreate(h, capG, defaultValue, flags));
  if (type == cudaGraphCondTypeWhile) {
    // a kernel in front of the node sets the condition every time the
    // enclosing graph reaches it: a loop inside another loop's body (the
    // PCG loop inside Newmark's Newton loop) would otherwise start from the
    // value that ended its previous run
    launch_set_condition((unsigned long long)*h, defaultValue, s);
    CUDA_TRY(cudaStreamGetCaptureInfo(s, &cs, nullptr, &capG, &deps, nullptr, &nd));
  }
  cudaGraphNodeParams p = {};
  p.type = cudaGraphNodeTypeConditional;
  p.conditional.handle = *h;
  p.conditional.type = type;
  p.conditional.size = size;
  cudaGraphNode_t node;
  CUDA_TRY(cudaGraphAddNode(&node, capG, deps, nullptr, nd, &p));
  for (unsigned k = 0; k < size; k++) bodies[k] = p.conditional.phGraph_out[k];
  CUDA_TRY(cudaStreamUpdateCaptureDependencies(s, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
  return HOBAK_OK;
}

// While-loop node on the capturing stream `s`.  Body: tile compaction, which
// also selects a grid class; a switch node whose bodies are the chunk of
// PCG iterations at each class's grid; k_continue, which keeps the loop
// going while any scene's inner PCG runs.
template <typename T>
int capture_pcg_loop(hobak_batch_t* B, cudaStream_t s, const PcgVecs<T>& v) {
  cudaGraphConditionalHandle hw, hs;
  cudaGraph_t body, cls[kGridClasses];
  if (int rc = add_conditional(s, cudaGraphCondTypeWhile, 1, 1, cudaGraphCondAssignDefault, &hw, &body)) return rc;
  CUDA_TRY(cudaStreamBeginCaptureToGraph(B->captureStream, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  const GridClasses gc = grid_classes(B->d.ntiles);
  int rc = HOBAK_OK;
  {
    // the switch handle belongs to the body graph, which is being captured
    cudaStreamCaptureStatus cs;
    cudaGraph_t capG = nullptr;
    CUDA_TRY(cudaStreamGetCaptureInfo(B->captureStream, &cs, nullptr, &capG, nullptr, nullptr, nullptr));
    CUDA_TRY(cudaGraphConditionalHandleCreate(&hs, capG, 0, 0));
  }
  launch_compact_tiles(B->d, B->captureStream, (unsigned long long)hs, &gc);
  {
    cudaStreamCaptureStatus cs;
    cudaGraph_t capG = nullptr;
    const cudaGraphNode_t* deps = nullptr;
    size_t nd = 0;
    CUDA_TRY(cudaStreamGetCaptureInfo(B->captureStream, &cs, nullptr, &capG, &deps, nullptr, &nd));
    cudaGraphNodeParams p = {};
    p.type = cudaGraphNodeTypeConditional;
    p.conditional.handle = hs;
    p.conditional.type = cudaGraphCondTypeSwitch;
    p.conditional.size = (unsigned)gc.n;
    cudaGraphNode_t node;
    CUDA_TRY(cudaGraphAddNode(&node, capG, deps, nullptr, nd, &p));
    for (int k = 0; k < gc.n; k++) cls[k] = p.conditional.phGraph_out[k];
    CUDA_TRY(cudaStreamUpdateCaptureDependencies(B->captureStream, &node, nullptr, 1,
                                                 cudaStreamSetCaptureDependencies));
  }
  for (int k = 0; k < gc.n && !rc; k++) {
    CUDA_TRY(cudaStreamBeginCaptureToGraph(B->captureStream2, cls[k], nullptr, nullptr, 0,
                                           cudaStreamCaptureModeThreadLocal));
    enqueue_chunk<T>(B->d, v, B->captureStream2, B->chunk, gc.grid[k]);
    cudaGraph_t out = nullptr;
    CUDA_TRY(cudaStreamEndCapture(B->captureStream2, &out));
  }
  launch_continue(B->d, (unsigned long long)hw, B->captureStream);
  cudaGraph_t out = nullptr;
  CUDA_TRY(cudaStreamEndCapture(B->captureStream, &out));
  return rc;
}

// Eager loop: compaction, then (host polls) the chunk at the grid class that
// covers the tiles left, until the device reports no running scene.
template <typename T>
int eager_pcg_loop(hobak_batch_t* B, cudaStream_t s, const PcgVecs<T>& v) {
  const GridClasses gc = grid_classes(B->d.ntiles);
  for (int iters = 0; iters <= B->opts.max_iters; iters += B->chunk) {
    launch_compact_tiles(B->d, s);
    CUDA_TRY(cudaMemcpyAsync(B->pinnedActive, B->d.active, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaMemcpyAsync(B->pinnedActive + 1, B->d.nLoopTiles, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(cudaStreamSynchronize(s));
    if (B->pinnedActive[0] <= 0) break;
    int k = 0;
    while (k + 1 < gc.n && gc.grid[k + 1] >= B->pinnedActive[1]) k++;
    enqueue_chunk<T>(B->d, v, s, B->chunk, gc.grid[k]);
    B->eagerChunks++;
  }
  return HOBAK_OK;
}

// The linear solve of a step: the cluster classes on their own streams, each
// launch solving its scenes to the end (mixed: every refinement sweep), beside
// the tile path's sweeps (an inner PCG and, mixed, the FP64 refinement);
// joined at the end.  Small scenes solve while large ones iterate, and a
// class's long-running scenes hold up neither the other classes nor the
// tile path's refinements.
template <typename T>
int enqueue_solve_t(hobak_batch_t* B, cudaStream_t s, bool capture, const PcgVecs<T>& v) {
  const DeviceBatch& d = B->d;
  const bool mixed = sizeof(T) == sizeof(float);
  const int sweeps = sweeps_of(B->opts);
  // the cluster classes solve their scenes completely, every sweep included
  // (cluster_pcg.cu), beside all of the tile path's sweeps
  int forked = 0;
  for (int c = kClusterClasses - 1; c >= 0; c--) {
    if (B->classes[c].count == 0) continue;
    if (!forked++) CUDA_TRY(cudaEventRecord(B->evFork, s));
    CUDA_TRY(cudaStreamWaitEvent(B->classStream[c], B->evFork, 0));
    const int ce = launch_cluster_pcg<T>(d, v, B->classes, c, B->classStream[c]);
    if (ce) return fail(HOBAK_ERR_CUDA, std::string("cluster PCG launch: ") + cudaGetErrorString((cudaError_t)ce));
    CUDA_TRY(cudaEventRecord(B->evJoin[c], B->classStream[c]));
  }
  for (int k = 0; k < sweeps && B->anyTileScene; k++) {
    launch_set_active(d, s);
    launch_inner_init<T>(d, v, s);
    int rc = capture ? capture_pcg_loop<T>(B, s, v) : eager_pcg_loop<T>(B, s, v);
    if (rc) return rc;
    if (mixed) launch_refine(d, s);
  }
  for (int c = 0; c < kClusterClasses; c++)
    if (B->classes[c].count) CUDA_TRY(cudaStreamWaitEvent(s, B->evJoin[c], 0));
  return HOBAK_OK;
}

// One Newton iteration of NEWMARK::solveRayleighDamped (NEWMARK.cpp:216-318):
// element terms at the current x, assembly, preconditioner, rhs and its
// |rhs|^2, the linear solve, x -= y and the per-scene Newton test.
template <typename T>
int enqueue_newton_body(hobak_batch_t* B, cudaStream_t s, bool capture, const PcgVecs<T>& v) {
  const DeviceBatch& d = B->d;
  if (sizeof(T) == sizeof(float)) launch_element_mixed(d, s);
  else launch_element(d, s);
  launch_green_damping(d, s);
  // contact at the iterate (NEWMARK.cpp:226-242)
  if (d.collOn) launch_collisions(d, d.coll, s);
  launch_assemble<T>(d, v, s);
  if (d.collOn) launch_collision_diag(d, d.coll, s);
  launch_diag_inverse<T>(d, v, B->opts.preconditioner, s);
  launch_rhs(d, s);
  if (int rc = enqueue_solve_t<T>(B, s, capture, v)) return rc;
  launch_newton_update(d, s);
  return HOBAK_OK;
}

// The Newton loop: a conditional WHILE node (graph) whose body ends in
// k_newton_continue, or a host loop over the same body (eager).
template <typename T>
int enqueue_newton_loop(hobak_batch_t* B, cudaStream_t s, bool capture, const PcgVecs<T>& v) {
  if (!capture) {
    for (int it = 0; it < B->opts.max_newton; it++) {
      if (int rc = enqueue_newton_body<T>(B, s, false, v)) return rc;
      B->eagerNewton++;
      CUDA_TRY(cudaMemcpyAsync(B->pinnedActive, B->d.newtonActive, sizeof(int), cudaMemcpyDeviceToHost, s));
      CUDA_TRY(cudaStreamSynchronize(s));
      if (B->pinnedActive[0] <= 0) break;
    }
    return HOBAK_OK;
  }
  cudaGraphConditionalHandle h;
  cudaGraph_t body;
  if (int rc = add_conditional(s, cudaGraphCondTypeWhile, 1, 1, cudaGraphCondAssignDefault, &h, &body)) return rc;
  CUDA_TRY(cudaStreamBeginCaptureToGraph(B->captureStreamN, body, nullptr, nullptr, 0,
                                         cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_newton_body<T>(B, B->captureStreamN, true, v);
  launch_newton_continue(B->d, (unsigned long long)h, B->captureStreamN);
  cudaGraph_t out = nullptr;
  CUDA_TRY(cudaStreamEndCapture(B->captureStreamN, &out));
  return rc;
}

// One step: BACKWARD_EULER_VELOCITY or BACKWARD_EULER_POSITION (element
// terms, assembly, preconditioner, rhs, the linear solve, update), or NEWMARK
// (the same inside a Newton loop).  `capture` builds the device-side loops of
// a graph; otherwise loops poll.  With `timed`, events bracket the phases
// (for Newmark the whole Newton loop is the solve phase: events cannot sit
// inside a conditional body).
template <typename T>
int enqueue_step_t(hobak_batch_t* B, cudaStream_t s, bool capture, bool timed, const PcgVecs<T>& v) {
  const DeviceBatch& d = B->d;
  const bool mixed = sizeof(T) == sizeof(float);
  const unsigned evFlags = capture ? cudaEventRecordExternal : cudaEventRecordDefault;
  if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[0], s, evFlags));
  launch_begin_step(d, s);
  if (B->opts.integrator == HOBAK_INTEGRATOR_NEWMARK) {
    launch_newton_begin(d, s);
    if (timed)
      for (int i = 1; i <= 3; i++) CUDA_TRY(cudaEventRecordWithFlags(B->ev[i], s, evFlags));
    if (int rc = enqueue_newton_loop<T>(B, s, capture, v)) return rc;
  } else {
    if (mixed) launch_element_mixed(d, s);
    else launch_element(d, s);
    if (d.collOn) launch_collisions(d, d.coll, s);
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[1], s, evFlags));
    launch_assemble<T>(d, v, s);
    if (d.collOn) launch_collision_diag(d, d.coll, s);
    launch_diag_inverse<T>(d, v, B->opts.preconditioner, s);
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[2], s, evFlags));
    launch_rhs(d, s);
    if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[3], s, evFlags));
    if (int rc = enqueue_solve_t<T>(B, s, capture, v)) return rc;
  }
  if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[4], s, evFlags));
  launch_finish_step(d, s);
  if (timed) CUDA_TRY(cudaEventRecordWithFlags(B->ev[5], s, evFlags));
  return HOBAK_OK;
}

int enqueue_step(hobak_batch_t* B, cudaStream_t s, bool capture, bool timed) {
  if (B->opts.precision == HOBAK_PRECISION_MIXED) return enqueue_step_t<float>(B, s, capture, timed, B->d.v32);
  return enqueue_step_t<double>(B, s, capture, timed, B->d.v64);
}

// The whole step as one graph (device-side while loops over PCG chunks), one
// instance per timing mode, built on first use.
int ensure_step_graph(hobak_batch_t* B, bool timed) {
  cudaGraphExec_t& exec = B->stepGraph[timed ? 1 : 0];
  if (exec) return HOBAK_OK;
  cudaGraph_t g = nullptr;
  CUDA_TRY(cudaStreamBeginCapture(B->stream, cudaStreamCaptureModeThreadLocal));
  int rc = enqueue_step(B, B->stream, true, timed);
  cudaError_t e = cudaStreamEndCapture(B->stream, &g);
  if (rc) {
    if (g) cudaGraphDestroy(g);
    return rc;
  }
  if (e != cudaSuccess) return fail(HOBAK_ERR_CUDA, std::string("step graph capture: ") + cudaGetErrorString(e));
  e = cudaGraphInstantiate(&exec, g, 0);
  cudaGraphDestroy(g);
  if (e != cudaSuccess) {
    exec = nullptr;
    return fail(HOBAK_ERR_CUDA, std::string("step graph instantiate: ") + cudaGetErrorString(e));
  }
  return HOBAK_OK;
}

void drop_graphs(hobak_batch_t* B) {
  for (auto& g : B->stepGraph)
    if (g) {
      cudaGraphExecDestroy(g);
      g = nullptr;
    }
}

// Surfaces of every scene (TET_MESH.cpp:294-350 order and winding, surface
// vertices 567-590, triangle neighbours 423-490, rest areas 494-525) and the
// device buffers of the per-step collision pipeline.
int build_collisions(hobak_batch_t* B) {
  const int n = (int)B->scenes.size();
  const auto& rest = B->restHost;
  B->surfTri.clear();
  B->svHost.clear();
  B->edgeHost.clear();
  B->surfTriStart.assign(1, 0);
  B->svStart.assign(1, 0);
  B->edgeStart.assign(1, 0);
  std::vector<int> triScene, triNbr, svScene, edgeScene, edgeTri;
  std::vector<double> triArea, svArea, edgeArea;
  auto area = [&](int a, int b2, int c) {
    double e1[3], e2[3];
    for (int i = 0; i < 3; i++) {
      e1[i] = rest[3 * (size_t)b2 + i] - rest[3 * (size_t)a + i];
      e2[i] = rest[3 * (size_t)c + i] - rest[3 * (size_t)a + i];
    }
    const double x = e1[1] * e2[2] - e1[2] * e2[1], y = e1[2] * e2[0] - e1[0] * e2[2], z = e1[0] * e2[1] - e1[1] * e2[0];
    return 0.5 * std::sqrt(x * x + y * y + z * z);
  };
  for (int s = 0; s < n; s++) {
    const SceneHost& H = B->scenes[s];
    // faces with their sorted keys; a face is on the surface if its key occurs once
    std::vector<std::array<int, 5>> keys;  // sorted triple, tet-local face index, position
    keys.reserve(4 * (size_t)H.nt);
    std::vector<std::array<int, 3>> faces(4 * (size_t)H.nt);
    for (int t = 0; t < H.nt; t++) {
      const int* v = &B->tetsHost[4 * (size_t)(H.t0 + t)];
      const std::array<int, 3> f[4] = {{v[0], v[1], v[3]}, {v[0], v[2], v[1]}, {v[0], v[3], v[2]}, {v[1], v[2], v[3]}};
      for (int k = 0; k < 4; k++) {
        faces[4 * (size_t)t + k] = f[k];
        std::array<int, 3> sk = f[k];
        std::sort(sk.begin(), sk.end());
        keys.push_back({sk[0], sk[1], sk[2], 0, 4 * t + k});
      }
    }
    std::sort(keys.begin(), keys.end());
    std::vector<char> surface(4 * (size_t)H.nt, 0);
    for (size_t i = 0; i < keys.size();) {
      size_t j = i;
      while (j < keys.size() && keys[j][0] == keys[i][0] && keys[j][1] == keys[i][1] && keys[j][2] == keys[i][2]) j++;
      if (j - i < 2) surface[keys[i][4]] = 1;
      i = j;
    }
    const int triBase = (int)B->surfTri.size() / 3;
    for (size_t k = 0; k < surface.size(); k++)
      if (surface[k]) {
        B->surfTri.insert(B->surfTri.end(), faces[k].begin(), faces[k].end());
        triScene.push_back(s);
      }
    const int ntri = (int)B->surfTri.size() / 3 - triBase;
    // surface vertices, ascending
    std::vector<int> sv;
    for (int k = 3 * triBase; k < 3 * (triBase + ntri); k++) sv.push_back(B->surfTri[k]);
    std::sort(sv.begin(), sv.end());
    sv.erase(std::unique(sv.begin(), sv.end()), sv.end());
    const int svBase = (int)B->svHost.size();
    B->svHost.insert(B->svHost.end(), sv.begin(), sv.end());
    svScene.insert(svScene.end(), sv.size(), s);
    svArea.resize(B->svHost.size(), 0.0);
    // neighbours across each edge (the other triangle sharing it)
    std::map<std::pair<int, int>, std::vector<int>> edges;
    for (int i = 0; i < ntri; i++)
      for (int j = 0; j < 3; j++) {
        int a = B->surfTri[3 * (triBase + i) + j], c = B->surfTri[3 * (triBase + i) + (j + 1) % 3];
        if (a > c) std::swap(a, c);
        edges[{a, c}].push_back(triBase + i);
      }
    for (int i = 0; i < ntri; i++) {
      const int f = triBase + i;
      for (int j = 0; j < 3; j++) {
        int a = B->surfTri[3 * f + j], c = B->surfTri[3 * f + (j + 1) % 3];
        if (a > c) std::swap(a, c);
        int nb = -1;
        for (int g : edges[{a, c}])
          if (g != f) nb = g;
        triNbr.push_back(nb);
      }
      const double A = area(B->surfTri[3 * f], B->surfTri[3 * f + 1], B->surfTri[3 * f + 2]);
      triArea.push_back(A);
      for (int j = 0; j < 3; j++) {
        const int v = B->surfTri[3 * f + j];
        const int id = svBase + int(std::lower_bound(sv.begin(), sv.end(), v) - sv.begin());
        svArea[id] += (1.0 / 3.0) * A;
      }
    }
    // surface edges (lo, hi) ascending (TET_MESH::computeSurfaceEdges,
    // TET_MESH.cpp:595-630), rest area = a third of each adjacent triangle's
    // in triangle order (TET_MESH.cpp:530-562), first two adjacent triangles
    // (computeSurfaceEdgeTriangleNeighbors, TET_MESH.cpp:356-412)
    {
      std::vector<std::array<int, 3>> ek;  // lo, hi, triangle
      for (int i = 0; i < ntri; i++)
        for (int j = 0; j < 3; j++) {
          int a = B->surfTri[3 * (triBase + i) + j], c = B->surfTri[3 * (triBase + i) + (j + 1) % 3];
          if (a > c) std::swap(a, c);
          ek.push_back({a, c, triBase + i});
        }
      std::sort(ek.begin(), ek.end());
      for (size_t i = 0; i < ek.size();) {
        size_t j = i;
        double A = 0.0;
        while (j < ek.size() && ek[j][0] == ek[i][0] && ek[j][1] == ek[i][1]) A += triArea[ek[j++][2]] / 3.0;
        B->edgeHost.push_back(ek[i][0]);
        B->edgeHost.push_back(ek[i][1]);
        edgeScene.push_back(s);
        edgeArea.push_back(A);
        edgeTri.push_back(ek[i][2]);
        edgeTri.push_back(j - i > 1 ? ek[i + 1][2] : -1);
        i = j;
      }
    }
    B->surfTriStart.push_back((int)B->surfTri.size() / 3);
    B->svStart.push_back((int)B->svHost.size());
    B->edgeStart.push_back((int)B->edgeHost.size() / 2);
  }
  const int nedge = (int)B->edgeHost.size() / 2;
  const int ntri = (int)B->surfTri.size() / 3, nsv = (int)B->svHost.size(), nv = B->nv;
  int hash = 1024;
  while (hash < 16 * std::max(ntri, 1)) hash <<= 1;
  const int cap = std::max(nsv * kMaxPairsPerVertex + nedge, 1);
  int eeHash = 1024;
  while (eeHash < 16 * std::max(nedge, 1)) eeHash <<= 1;
  const int scanBlocks = (std::max(std::max(std::max(hash, nsv), nv), std::max(nedge, eeHash)) + 1023) / 1024 + 1;
  Arena A;
  const size_t oScenes = A.reserve(sizeof(CollisionScene) * n);
  const size_t oTri = A.reserve(sizeof(int) * 3 * (size_t)ntri), oTriScene = A.reserve(sizeof(int) * ntri);
  const size_t oTriArea = A.reserve(sizeof(double) * ntri), oTriNbr = A.reserve(sizeof(int) * 3 * (size_t)ntri);
  const size_t oSv = A.reserve(sizeof(int) * nsv), oSvScene = A.reserve(sizeof(int) * nsv);
  const size_t oSvArea = A.reserve(sizeof(double) * nsv);
  const size_t oCell = A.reserve(sizeof(unsigned) * n), oInv = A.reserve(nv), oSkip = A.reserve(ntri);
  const size_t oBucket = A.reserve(sizeof(int) * (hash + 1)), oCursor = A.reserve(sizeof(int) * hash);
  const size_t oEntry = A.reserve(sizeof(int) * 8 * (size_t)ntri);
  const size_t oSvCount = A.reserve(sizeof(int) * (nsv + 1));
  const size_t oCand = A.reserve(sizeof(int) * (size_t)kMaxPairsPerVertex * nsv);
  const size_t oOver = A.reserve(sizeof(int)), oNp = A.reserve(sizeof(int));
  const size_t oPairTet = A.reserve(sizeof(int4) * (size_t)cap), oPairC = A.reserve(sizeof(double) * 4 * (size_t)cap);
  const size_t oPairG = A.reserve(sizeof(double) * 9 * (size_t)cap);
  const size_t oPairR = A.reserve(sizeof(double) * 12 * (size_t)cap);
  const size_t oPairF = A.reserve(sizeof(double) * 12 * (size_t)cap);
  const size_t oDiag = A.reserve(sizeof(double) * 9 * (size_t)nv);
  const size_t oIncCount = A.reserve(sizeof(int) * (nv + 1)), oIncCursor = A.reserve(sizeof(int) * nv);
  const size_t oIncList = A.reserve(sizeof(int) * 4 * (size_t)cap);
  const size_t oScan = A.reserve(sizeof(int) * scanBlocks);
  const size_t oEdge = A.reserve(sizeof(int2) * (size_t)nedge), oEdgeScene = A.reserve(sizeof(int) * nedge);
  const size_t oEdgeArea = A.reserve(sizeof(double) * nedge), oEdgeTri = A.reserve(sizeof(int2) * (size_t)nedge);
  const size_t oEeSel = A.reserve(sizeof(int) * nedge), oEeKeep = A.reserve(nedge), oEeCross = A.reserve(nedge);
  const size_t oEeAB = A.reserve(sizeof(double4) * (size_t)nedge), oEeCount = A.reserve(sizeof(int) * (nedge + 1));
  const size_t oEeCell = A.reserve(sizeof(unsigned) * n), oEeBucket = A.reserve(sizeof(int) * (eeHash + 1));
  const size_t oEeCursor = A.reserve(sizeof(int) * eeHash), oEeEntry = A.reserve(sizeof(int) * 8 * (size_t)nedge);
  void* base = nullptr;
  cudaError_t e = cudaMalloc(&base, A.used);
  if (e != cudaSuccess)
    return fail(e == cudaErrorMemoryAllocation ? HOBAK_ERR_NO_MEMORY : HOBAK_ERR_CUDA,
                std::string("cudaMalloc of collision buffers: ") + cudaGetErrorString(e));
  B->collArena = base;
  B->collBytes = A.used;
  CUDA_TRY(cudaMemset(base, 0, A.used));
  DeviceCollisions& c = B->d.coll;
  c.nscenes = n;
  c.ntri = ntri;
  c.nsv = nsv;
  c.nv = nv;
  c.hashSize = hash;
  c.pairCap = cap;
  c.scenes = carve<CollisionScene>(base, oScenes);
  c.tri = carve<int>(base, oTri);
  c.triScene = carve<int>(base, oTriScene);
  c.triArea = carve<double>(base, oTriArea);
  c.triNbr = carve<int>(base, oTriNbr);
  c.sv = carve<int>(base, oSv);
  c.svScene = carve<int>(base, oSvScene);
  c.svArea = carve<double>(base, oSvArea);
  c.cellBits = carve<unsigned>(base, oCell);
  c.vInverted = carve<unsigned char>(base, oInv);
  c.triSkip = carve<unsigned char>(base, oSkip);
  c.bucketCount = carve<int>(base, oBucket);
  c.bucketCursor = carve<int>(base, oCursor);
  c.entryTri = carve<int>(base, oEntry);
  c.svCount = carve<int>(base, oSvCount);
  c.svCand = carve<int>(base, oCand);
  c.overflow = carve<int>(base, oOver);
  c.npairs = carve<int>(base, oNp);
  c.pairTet = carve<int4>(base, oPairTet);
  c.pairC = carve<double>(base, oPairC);
  c.pairG = carve<double>(base, oPairG);
  c.pairRhs = carve<double>(base, oPairR);
  c.pairF = carve<double>(base, oPairF);
  c.diag = carve<double>(base, oDiag);
  c.incCount = carve<int>(base, oIncCount);
  c.incCursor = carve<int>(base, oIncCursor);
  c.incList = carve<int>(base, oIncList);
  c.scanTmp = carve<int>(base, oScan);
  c.nedge = nedge;
  c.edge = carve<int2>(base, oEdge);
  c.edgeScene = carve<int>(base, oEdgeScene);
  c.edgeArea = carve<double>(base, oEdgeArea);
  c.edgeTri = carve<int2>(base, oEdgeTri);
  c.eeSel = carve<int>(base, oEeSel);
  c.eeKeep = carve<unsigned char>(base, oEeKeep);
  c.eeCross = carve<unsigned char>(base, oEeCross);
  c.eeAB = carve<double4>(base, oEeAB);
  c.eeCount = carve<int>(base, oEeCount);
  c.eeHashSize = eeHash;
  c.eeCellBits = carve<unsigned>(base, oEeCell);
  c.eeBucketCount = carve<int>(base, oEeBucket);
  c.eeBucketCursor = carve<int>(base, oEeCursor);
  c.eeEntry = carve<int>(base, oEeEntry);
  B->collScenes.assign(n, CollisionScene{0, 0, 0, 0, 0, 0.01, 1.0, 0.001});
  for (int s = 0; s < n; s++) {
    B->collScenes[s].tri0 = B->surfTriStart[s];
    B->collScenes[s].ntri = B->surfTriStart[s + 1] - B->surfTriStart[s];
    B->collScenes[s].sv0 = B->svStart[s];
    B->collScenes[s].nsv = B->svStart[s + 1] - B->svStart[s];
    B->collScenes[s].e0 = B->edgeStart[s];
    B->collScenes[s].ne = B->edgeStart[s + 1] - B->edgeStart[s];
  }
  auto up = [&](const void* dst, const void* src, size_t bytes) {
    return bytes ? cudaMemcpy(const_cast<void*>(dst), src, bytes, cudaMemcpyHostToDevice) : cudaSuccess;
  };
  CUDA_TRY(up(c.scenes, B->collScenes.data(), sizeof(CollisionScene) * n));
  CUDA_TRY(up(c.tri, B->surfTri.data(), sizeof(int) * B->surfTri.size()));
  CUDA_TRY(up(c.triScene, triScene.data(), sizeof(int) * triScene.size()));
  CUDA_TRY(up(c.triArea, triArea.data(), sizeof(double) * triArea.size()));
  CUDA_TRY(up(c.triNbr, triNbr.data(), sizeof(int) * triNbr.size()));
  CUDA_TRY(up(c.sv, B->svHost.data(), sizeof(int) * B->svHost.size()));
  CUDA_TRY(up(c.svScene, svScene.data(), sizeof(int) * svScene.size()));
  CUDA_TRY(up(c.svArea, svArea.data(), sizeof(double) * svArea.size()));
  if (nedge > 0) {
    CUDA_TRY(up(c.edge, B->edgeHost.data(), sizeof(int2) * (size_t)nedge));
    CUDA_TRY(up(c.edgeScene, edgeScene.data(), sizeof(int) * nedge));
    CUDA_TRY(up(c.edgeArea, edgeArea.data(), sizeof(double) * nedge));
    CUDA_TRY(up(c.edgeTri, edgeTri.data(), sizeof(int2) * (size_t)nedge));
  }
  B->d.collOn = 1;
  return HOBAK_OK;
}

// Enqueue nsteps steps; with graphs nothing waits on the host in between.
int run_steps(hobak_batch_t* B, int nsteps) {
  cudaStream_t s = B->stream;
  const bool timed = B->timing;
  if (int rc = prepare_cluster_classes(B)) return rc;
  if (int rc = reorder_cluster_classes(B)) return rc;
  // cleared once per call: an overflow in any step or Newton iteration is reported
  if (B->d.collOn) CUDA_TRY(cudaMemsetAsync(B->d.coll.overflow, 0, sizeof(int), s));
  for (int k = 0; k < nsteps; k++) {
    if (B->opts.use_graph) {
      int rc = ensure_step_graph(B, timed);
      if (rc) return rc;
      CUDA_TRY(cudaGraphLaunch(B->stepGraph[timed ? 1 : 0], s));
    } else {
      int rc = enqueue_step(B, s, false, timed);
      if (rc) return rc;
    }
    B->launches += fixed_launches(B);
    const int elaunch = element_launches(B->d, B->opts.precision == HOBAK_PRECISION_MIXED);
    B->phaseLaunches[0] += 1 + elaunch;
    B->phaseLaunches[1] += 2;
    B->phaseLaunches[2] += 1;
    B->phaseLaunches[3] += fixed_launches(B) - 5 - elaunch - (B->d.collOn ? collision_launches(B->d.coll) : 0);
    if (B->d.collOn) B->phaseLaunches[0] += collision_launches(B->d.coll);
    B->phaseLaunches[4] += 1;
    if (timed) {
      CUDA_TRY(cudaEventSynchronize(B->ev[5]));
      for (int i = 0; i < 5; i++) {
        float ms = 0;
        CUDA_TRY(cudaEventElapsedTime(&ms, B->ev[i], B->ev[i + 1]));
        B->phaseMs[i] += ms;
      }
    }
  }
  CUDA_TRY(cudaGetLastError());
  return HOBAK_OK;
}

// Loop-body kernels launched so far (device counter of loop-body runs, or
// the host count of eager chunks).
int count_loop_launches(hobak_batch_t* B, long long* out) {
  unsigned long long runs = 0;
  CUDA_TRY(cudaMemcpy(&runs, B->d.bodyRuns, sizeof(runs), cudaMemcpyDeviceToHost));
  // a loop body = tile compaction + chunk x (SpMV, update) + k_continue; an
  // eager chunk has no k_continue
  *out = B->loopLaunchBase + (long long)(runs * (2ull * B->chunk + 2ull)) + B->eagerChunks * (2LL * B->chunk + 1);
  // Newmark's Newton loop bodies (graph: with k_newton_continue)
  unsigned long long nruns = 0;
  CUDA_TRY(cudaMemcpy(&nruns, B->d.newtonRuns, sizeof(nruns), cudaMemcpyDeviceToHost));
  *out += (long long)nruns * (newton_body_launches(B) + 1) + B->eagerNewton * newton_body_launches(B);
  return HOBAK_OK;
}

// Before the chunk size changes: fold the loop launches counted so far into
// the base and restart the counters.
int fold_loop_launches(hobak_batch_t* B) {
  long long n = 0;
  int rc = count_loop_launches(B, &n);
  if (rc) return rc;
  B->loopLaunchBase = n;
  B->eagerChunks = 0;
  CUDA_TRY(cudaMemset(B->d.bodyRuns, 0, sizeof(unsigned long long)));
  CUDA_TRY(cudaMemset(B->d.newtonRuns, 0, sizeof(unsigned long long)));
  B->eagerNewton = 0;
  return HOBAK_OK;
}

// Tiles of TV consecutive vertices of one scene (one PCG CTA each): host
// tables, scene ranges, device upload.  Graphs are dropped (they hold the
// launch shapes).
int apply_tile_size(hobak_batch_t* B, int TV) {
  if (TV != 64 && TV != 128) return fail(HOBAK_ERR_INVALID, "tile size must be 64 or 128 vertices");
  std::vector<int> tileScene, tileV0, tileV1;
  for (int s = 0; s < (int)B->scenes.size(); s++) {
    SceneHost& H = B->scenes[s];
    H.tile0 = (int)tileScene.size();
    for (int u = 0; u < H.nv; u += TV) {
      tileScene.push_back(s);
      tileV0.push_back(H.v0 + u);
      tileV1.push_back(H.v0 + std::min(H.nv, u + TV));
    }
    H.ntiles = (int)tileScene.size() - H.tile0;
    B->sceneParams[s].tile0 = H.tile0;
    B->sceneParams[s].ntiles = H.ntiles;
  }
  const int ntiles = (int)tileScene.size();
  if (ntiles > B->ntilesCap) return fail(HOBAK_ERR_INVALID, "tile tables too small");
  DeviceBatch& d = B->d;
  CUDA_TRY(cudaStreamSynchronize(B->stream));
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(d.scenes), B->sceneParams.data(),
                      sizeof(SceneParams) * B->sceneParams.size(), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(const_cast<int*>(d.tileScene), tileScene.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(const_cast<int*>(d.tileV0), tileV0.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(const_cast<int*>(d.tileV1), tileV1.data(), sizeof(int) * ntiles, cudaMemcpyHostToDevice));
  d.ntiles = ntiles;
  d.tileV = TV;
  B->ntiles = ntiles;
  drop_graphs(B);
  return HOBAK_OK;
}

}  // namespace

// ---------------------------------------------------------------------------
extern "C" {

const char* hobak_version(void) { return "hobak-gb300 0.1 (sm_103a)"; }

const char* hobak_last_error(void) { return g_lastError.c_str(); }

int hobak_device_check(int* major, int* minor, int* sms) {
  int dev = 0;
  cudaDeviceProp p;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(HOBAK_ERR_NO_DEVICE, std::string("no CUDA device: ") + cudaGetErrorString(e));
  e = cudaGetDeviceProperties(&p, dev);
  if (e != cudaSuccess) return fail(HOBAK_ERR_NO_DEVICE, cudaGetErrorString(e));
  if (major) *major = p.major;
  if (minor) *minor = p.minor;
  if (sms) *sms = p.multiProcessorCount;
  if (p.major != 10) return fail(HOBAK_ERR_NO_DEVICE, "this build targets sm_103a (Blackwell Ultra) only");
  return HOBAK_OK;
}

void hobak_default_solver_opts(hobak_solver_opts* o) {
  if (!o) return;
  o->tol = 1e-8;
  o->max_iters = 1000;
  o->precision = HOBAK_PRECISION_FP64;
  o->preconditioner = HOBAK_PRECOND_BLOCK_JACOBI;
  o->max_refinements = 3;
  o->use_graph = 1;
  o->integrator = HOBAK_INTEGRATOR_VELOCITY;
  o->rayleigh_alpha = 0.01;
  o->rayleigh_beta = 0.01;
  o->max_newton = 10;           // NEWMARK.cpp:41
  o->newton_tolerance = 1e-7;   // NEWMARK.cpp:43
  o->inner_tolerance = 1e-5;
}

int hobak_batch_create(const hobak_scene_desc* scenes, int nscenes, const hobak_solver_opts* opts,
                       hobak_batch* out) {
  if (!out) return fail(HOBAK_ERR_INVALID, "null output handle");
  *out = nullptr;
  if (!scenes || nscenes <= 0) return fail(HOBAK_ERR_INVALID, "no scenes");
  int rc = check_opts(opts);
  if (rc) return rc;
  for (int s = 0; s < nscenes; s++)
    if ((rc = validate_scene(scenes[s], s))) return rc;
  if ((rc = hobak_device_check(nullptr, nullptr, nullptr))) return rc;
  std::unique_ptr<hobak_batch_t> B(new hobak_batch_t);
  if (opts)
    B->opts = *opts;
  else
    hobak_default_solver_opts(&B->opts);
  CUDA_TRY(cudaStreamCreateWithFlags(&B->stream, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&B->captureStream, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&B->captureStream2, cudaStreamNonBlocking));
  CUDA_TRY(cudaStreamCreateWithFlags(&B->captureStreamN, cudaStreamNonBlocking));
  for (auto& cs : B->classStream) CUDA_TRY(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
  CUDA_TRY(cudaEventCreateWithFlags(&B->evFork, cudaEventDisableTiming));
  for (auto& e : B->evJoin) CUDA_TRY(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  CUDA_TRY(cudaMallocHost(&B->pinnedActive, 2 * sizeof(int)));
  CUDA_TRY(cudaMallocHost(&B->solvePinned, sizeof(SolveState) * nscenes));
  for (auto& e : B->ev) CUDA_TRY(cudaEventCreate(&e));
  if ((rc = build_batch(B.get(), scenes, nscenes))) {
    hobak_batch_destroy(B.release());
    return rc;
  }
  if (B->opts.integrator == HOBAK_INTEGRATOR_POSITION && (rc = rest_hessian(B.get()))) {
    hobak_batch_destroy(B.release());
    return rc;
  }
  if ((rc = upload_solver_opts(B.get()))) {
    hobak_batch_destroy(B.release());
    return rc;
  }
  *out = B.release();
  return HOBAK_OK;
}

int hobak_batch_destroy(hobak_batch b) {
  if (!b) return HOBAK_OK;
  if (b->collArena) cudaFree(b->collArena);
  drop_graphs(b);
  if (b->captureStream) cudaStreamDestroy(b->captureStream);
  if (b->captureStream2) cudaStreamDestroy(b->captureStream2);
  if (b->captureStreamN) cudaStreamDestroy(b->captureStreamN);
  for (auto& cs : b->classStream)
    if (cs) cudaStreamDestroy(cs);
  if (b->evFork) cudaEventDestroy(b->evFork);
  for (auto& e : b->evJoin)
    if (e) cudaEventDestroy(e);
  for (auto& e : b->ev)
    if (e) cudaEventDestroy(e);
  if (b->pinnedActive) cudaFreeHost(b->pinnedActive);
  if (b->solvePinned) cudaFreeHost(b->solvePinned);
  if (b->arena) cudaFree(b->arena);
  if (b->precArena) cudaFree(b->precArena);
  if (b->K0) cudaFree(b->K0);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
  return HOBAK_OK;
}

int hobak_batch_num_scenes(hobak_batch b, int* n) {
  if (!b || !n) return fail(HOBAK_ERR_INVALID, "null handle");
  *n = (int)b->scenes.size();
  return HOBAK_OK;
}

int hobak_batch_step_async(hobak_batch b, int nsteps) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  if (nsteps < 0) return fail(HOBAK_ERR_INVALID, "nsteps < 0");
  int rc = run_steps(b, nsteps);
  if (rc) return rc;
  const int n = (int)b->scenes.size();
  CUDA_TRY(cudaMemcpyAsync(b->solvePinned, b->d.solve, sizeof(SolveState) * n, cudaMemcpyDeviceToHost, b->stream));
  b->pending = true;
  return HOBAK_OK;
}

int hobak_batch_query(hobak_batch b) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  const cudaError_t e = cudaStreamQuery(b->stream);
  if (e == cudaSuccess) return 1;
  if (e == cudaErrorNotReady) return 0;
  return fail(HOBAK_ERR_CUDA, std::string("cudaStreamQuery: ") + cudaGetErrorString(e));
}

int hobak_batch_step(hobak_batch b, int nsteps, hobak_step_stats* stats) {
  int rc = hobak_batch_step_async(b, nsteps);
  if (rc) return rc;
  return hobak_batch_wait(b, stats);
}

int hobak_batch_wait(hobak_batch b, hobak_step_stats* stats) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  const int n = (int)b->scenes.size();
  if (b->pending) {
    b->lastSolve.assign(b->solvePinned, b->solvePinned + n);
    b->pending = false;
    b->clusterOrderStale = true;
  }
  if ((int)b->lastSolve.size() != n) return HOBAK_OK;  // nothing stepped yet
  int status = HOBAK_OK;
  for (int s = 0; s < n; s++) {
    const SolveState& st = b->lastSolve[s];
    if (st.converged < 0) status = HOBAK_ERR_NAN;
    else if (st.converged == 0 && status == HOBAK_OK) status = HOBAK_WARN_NOT_CONVERGED;
    if (stats) {
      stats[s].iterations = st.totalIters;
      stats[s].converged = st.converged > 0 ? 1 : 0;
      stats[s].rel_residual = st.rhsNorm2 > 0 ? std::sqrt(st.rr64 / st.rhsNorm2) : 0.0;
      stats[s].refinements = st.sweep > 0 ? st.sweep - 1 : 0;
    }
  }
  if (status == HOBAK_ERR_NAN) return fail(status, "non-finite residual in PCG");
  if (b->d.collOn) {
    int over = 0;
    CUDA_TRY(cudaMemcpy(&over, b->d.coll.overflow, sizeof(int), cudaMemcpyDeviceToHost));
    if (over)
      return fail(HOBAK_ERR_OVERFLOW, "a surface vertex had more than 16 vertex-face candidates; contacts were dropped");
  }
  return status;
}

int hobak_batch_set_state(hobak_batch b, int scene, const double* x, const double* v) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  const SceneHost& H = b->scenes[scene];
  const size_t bytes = 3 * sizeof(double) * H.nv;
  if (x) CUDA_TRY(cudaMemcpyAsync(b->d.x + 3 * (size_t)H.v0, x, bytes, cudaMemcpyHostToDevice, b->stream));
  if (v) CUDA_TRY(cudaMemcpyAsync(b->d.v + 3 * (size_t)H.v0, v, bytes, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_get_state(hobak_batch b, int scene, double* x, double* v) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  const SceneHost& H = b->scenes[scene];
  const size_t bytes = 3 * sizeof(double) * H.nv;
  if (x) CUDA_TRY(cudaMemcpyAsync(x, b->d.x + 3 * (size_t)H.v0, bytes, cudaMemcpyDeviceToHost, b->stream));
  if (v) CUDA_TRY(cudaMemcpyAsync(v, b->d.v + 3 * (size_t)H.v0, bytes, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_get_acceleration(hobak_batch b, int scene, double* a) {
  if (!b || !a || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const SceneHost& H = b->scenes[scene];
  CUDA_TRY(cudaMemcpyAsync(a, b->d.acc + 3 * (size_t)H.v0, 3 * sizeof(double) * H.nv, cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_set_acceleration(hobak_batch b, int scene, const double* a) {
  if (!b || !a || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const SceneHost& H = b->scenes[scene];
  CUDA_TRY(cudaMemcpyAsync(b->d.acc + 3 * (size_t)H.v0, a, 3 * sizeof(double) * H.nv, cudaMemcpyHostToDevice,
                           b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_set_pin_targets(hobak_batch b, int scene, const double* targets) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  const SceneHost& H = b->scenes[scene];
  if (H.pinned.empty()) return HOBAK_OK;
  if (!targets) return fail(HOBAK_ERR_INVALID, "null targets");
  for (size_t k = 0; k < H.pinned.size(); k++)
    for (int i = 0; i < 3; i++) {
      const double t = targets[3 * k + i];
      if (!std::isfinite(t)) return fail(HOBAK_ERR_INVALID, "non-finite pin target");
      b->pinTargetHost[3 * (size_t)H.pinned[k] + i] = t;
    }
  // the scene's range in one copy; the step graph reads the targets from HBM
  const size_t q0 = 3 * (size_t)H.v0;
  CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(b->d.pinTarget) + q0, b->pinTargetHost.data() + q0,
                           3 * sizeof(double) * H.nv, cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

// Snapshot layout: a 64-byte header, then x, v, acceleration, external
// forces and pin targets (3 * total vertices doubles each, scenes back to
// back) and one active byte per scene.
namespace {
constexpr unsigned kSnapshotMagic = 0x534b4248u;  // "HBKS"
constexpr int kSnapshotVersion = 1;
constexpr int kSnapshotArrays = 5;
struct SnapshotHeader {
  unsigned magic;
  int version, nscenes, nv;
  unsigned long long vertexHash;  // FNV-1a over the per-scene vertex counts
  unsigned char pad[40];
};
static_assert(sizeof(SnapshotHeader) == 64, "snapshot header is 64 bytes");

unsigned long long scene_shape_hash(const hobak_batch_t* b) {
  unsigned long long h = 1469598103934665603ull;
  for (const SceneHost& H : b->scenes) {
    h ^= (unsigned long long)(unsigned)H.nv;
    h *= 1099511628211ull;
  }
  return h;
}

size_t snapshot_bytes(const hobak_batch_t* b) {
  return sizeof(SnapshotHeader) + kSnapshotArrays * 3 * sizeof(double) * (size_t)b->nv + b->scenes.size();
}
}  // namespace

int hobak_batch_snapshot_bytes(hobak_batch b, size_t* bytes) {
  if (!b || !bytes) return fail(HOBAK_ERR_INVALID, "bad arguments");
  *bytes = snapshot_bytes(b);
  return HOBAK_OK;
}

int hobak_batch_snapshot(hobak_batch b, void* dst, size_t bytes) {
  if (!b || !dst) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (bytes < snapshot_bytes(b)) return fail(HOBAK_ERR_INVALID, "snapshot buffer too small");
  SnapshotHeader h{};
  h.magic = kSnapshotMagic;
  h.version = kSnapshotVersion;
  h.nscenes = (int)b->scenes.size();
  h.nv = b->nv;
  h.vertexHash = scene_shape_hash(b);
  std::vector<unsigned char> active(b->scenes.size());
  for (size_t i = 0; i < active.size(); i++) active[i] = b->sceneParams[i].active ? 1 : 0;
  const size_t V3 = 3 * sizeof(double) * (size_t)b->nv;
  unsigned char* p = static_cast<unsigned char*>(dst);
  // cudaMemcpyDefault: dst may be host (pageable or pinned) or device memory
  CUDA_TRY(cudaMemcpyAsync(p, &h, sizeof(h), cudaMemcpyDefault, b->stream));
  p += sizeof(h);
  const double* src[kSnapshotArrays] = {b->d.x, b->d.v, b->d.acc, b->d.fext, b->d.pinTarget};
  for (int k = 0; k < kSnapshotArrays; k++, p += V3)
    CUDA_TRY(cudaMemcpyAsync(p, src[k], V3, cudaMemcpyDefault, b->stream));
  CUDA_TRY(cudaMemcpyAsync(p, active.data(), active.size(), cudaMemcpyDefault, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_restore(hobak_batch b, const void* src, size_t bytes) {
  if (!b || !src) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (bytes < snapshot_bytes(b)) return fail(HOBAK_ERR_INVALID, "snapshot too small for this batch");
  SnapshotHeader h{};
  CUDA_TRY(cudaMemcpy(&h, src, sizeof(h), cudaMemcpyDefault));
  if (h.magic != kSnapshotMagic || h.version != kSnapshotVersion) return fail(HOBAK_ERR_INVALID, "not a snapshot");
  if (h.nscenes != (int)b->scenes.size() || h.nv != b->nv || h.vertexHash != scene_shape_hash(b))
    return fail(HOBAK_ERR_INVALID, "snapshot of a batch with other scenes");
  const size_t V3 = 3 * sizeof(double) * (size_t)b->nv;
  const unsigned char* p = static_cast<const unsigned char*>(src) + sizeof(h);
  double* dstArr[kSnapshotArrays] = {b->d.x, b->d.v, b->d.acc, const_cast<double*>(b->d.fext),
                                     const_cast<double*>(b->d.pinTarget)};
  for (int k = 0; k < kSnapshotArrays; k++, p += V3)
    CUDA_TRY(cudaMemcpyAsync(dstArr[k], p, V3, cudaMemcpyDefault, b->stream));
  std::vector<unsigned char> active(b->scenes.size());
  CUDA_TRY(cudaMemcpyAsync(active.data(), p, active.size(), cudaMemcpyDefault, b->stream));
  CUDA_TRY(cudaMemcpyAsync(b->pinTargetHost.data(), b->d.pinTarget, V3, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  for (size_t i = 0; i < active.size(); i++)
    if ((b->sceneParams[i].active != 0) != (active[i] != 0))
      if (int rc = hobak_batch_set_active(b, (int)i, active[i])) return rc;
  return HOBAK_OK;
}

// Whole-batch state: every scene's 3*nv values back to back in scene order,
// which is how the batch keeps them on the device, so each is one copy.
int hobak_batch_set_state_all(hobak_batch b, const double* x, const double* v) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  const size_t bytes = 3 * sizeof(double) * (size_t)b->nv;
  if (x) CUDA_TRY(cudaMemcpyAsync(b->d.x, x, bytes, cudaMemcpyHostToDevice, b->stream));
  if (v) CUDA_TRY(cudaMemcpyAsync(b->d.v, v, bytes, cudaMemcpyHostToDevice, b->stream));
  return HOBAK_OK;
}

int hobak_batch_get_state_all(hobak_batch b, double* x, double* v) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  const size_t bytes = 3 * sizeof(double) * (size_t)b->nv;
  if (x) CUDA_TRY(cudaMemcpyAsync(x, b->d.x, bytes, cudaMemcpyDeviceToHost, b->stream));
  if (v) CUDA_TRY(cudaMemcpyAsync(v, b->d.v, bytes, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_set_external_forces_all(hobak_batch b, const double* f) {
  if (!b || !f) return fail(HOBAK_ERR_INVALID, "bad arguments");
  CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(b->d.fext), f, 3 * sizeof(double) * (size_t)b->nv,
                           cudaMemcpyHostToDevice, b->stream));
  return HOBAK_OK;
}

int hobak_batch_set_external_forces(hobak_batch b, int scene, const double* f) {
  if (!b || !f || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const SceneHost& H = b->scenes[scene];
  CUDA_TRY(cudaMemcpyAsync(const_cast<double*>(b->d.fext) + 3 * (size_t)H.v0, f, 3 * sizeof(double) * H.nv,
                           cudaMemcpyHostToDevice, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

int hobak_batch_set_solver(hobak_batch b, const hobak_solver_opts* opts) {
  if (!b || !opts) return fail(HOBAK_ERR_INVALID, "bad arguments");
  int rc = check_opts(opts);
  if (rc) return rc;
  b->opts = *opts;
  b->clusterDirty = true;
  drop_graphs(b);
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if ((opts->precision == HOBAK_PRECISION_MIXED) != b->precMixed) {
    if ((rc = alloc_precision(b))) return rc;
  }
  for (SceneParams& p : b->sceneParams) set_integrator(p, *opts);
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(b->d.scenes), b->sceneParams.data(),
                      sizeof(SceneParams) * b->sceneParams.size(), cudaMemcpyHostToDevice));
  if (opts->integrator == HOBAK_INTEGRATOR_POSITION && (rc = rest_hessian(b))) return rc;
  return upload_solver_opts(b);
}

int hobak_batch_set_collisions(hobak_batch b, int scene, int vf_on, double eps, double stiffness,
                               double damping_beta) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (vf_on && !(eps > 0.0)) return fail(HOBAK_ERR_INVALID, "collision distance must be > 0");
  if (!b->collArena) {
    int rc = build_collisions(b);
    if (rc) return rc;
  }
  CollisionScene& cs = b->collScenes[scene];
  cs.vfOn = vf_on ? 1 : 0;
  cs.eps = eps;
  cs.mu = stiffness;
  cs.beta = damping_beta;
  std::vector<CollisionScene> eff = b->collScenes;
  for (size_t k = 0; k < eff.size(); k++)
    if (!b->sceneParams[k].active) eff[k].vfOn = eff[k].eeOn = 0;
  CUDA_TRY(cudaMemcpy(const_cast<CollisionScene*>(b->d.coll.scenes), eff.data(), sizeof(CollisionScene) * eff.size(),
                      cudaMemcpyHostToDevice));
  b->clusterDirty = true;
  drop_graphs(b);
  return HOBAK_OK;
}

int hobak_batch_set_edge_collisions(hobak_batch b, int scene, int ee_on) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (!b->collArena) {
    int rc = build_collisions(b);
    if (rc) return rc;
  }
  CollisionScene& cs = b->collScenes[scene];
  if (ee_on && !(cs.eps > 0.0)) return fail(HOBAK_ERR_INVALID, "collision distance must be > 0");
  cs.eeOn = ee_on ? 1 : 0;
  CollisionScene eff = cs;
  if (!b->sceneParams[scene].active) eff.vfOn = eff.eeOn = 0;
  CUDA_TRY(cudaMemcpy(const_cast<CollisionScene*>(b->d.coll.scenes) + scene, &eff, sizeof(CollisionScene),
                      cudaMemcpyHostToDevice));
  b->clusterDirty = true;
  drop_graphs(b);
  return HOBAK_OK;
}

int hobak_batch_edge_pairs(hobak_batch b, int scene, int* npairs, int* quads, int cap) {
  if (!b || !npairs || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad arguments");
  *npairs = 0;
  if (!b->collArena) return HOBAK_OK;
  const int e0 = b->edgeStart[scene], e1 = b->edgeStart[scene + 1], ne = e1 - e0;
  if (ne == 0) return HOBAK_OK;
  std::vector<int> sel(ne);
  std::vector<unsigned char> keep(ne);
  CUDA_TRY(cudaMemcpyAsync(sel.data(), b->d.coll.eeSel + e0, sizeof(int) * ne, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaMemcpyAsync(keep.data(), b->d.coll.eeKeep + e0, ne, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  const int v0 = b->scenes[scene].v0;
  int n = 0;
  for (int x = 0; x < ne; x++) {
    if (!keep[x]) continue;
    if (quads && n < cap) {
      const int y = sel[x];
      quads[4 * n] = b->edgeHost[2 * (e0 + x)] - v0;
      quads[4 * n + 1] = b->edgeHost[2 * (e0 + x) + 1] - v0;
      quads[4 * n + 2] = b->edgeHost[2 * y] - v0;
      quads[4 * n + 3] = b->edgeHost[2 * y + 1] - v0;
    }
    n++;
  }
  *npairs = n;
  return HOBAK_OK;
}

int hobak_batch_collision_pairs(hobak_batch b, int scene, int detect_now, int* npairs, int* pairs, int cap,
                                int* ntris, int* tris) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (!b->collArena) {
    int rc = build_collisions(b);
    if (rc) return rc;
  }
  const SceneHost& H = b->scenes[scene];
  const int t0 = b->surfTriStart[scene], t1 = b->surfTriStart[scene + 1];
  const int s0 = b->svStart[scene], s1 = b->svStart[scene + 1];
  if (ntris) *ntris = t1 - t0;
  if (tris)
    for (int k = 3 * t0; k < 3 * t1; k++) tris[k - 3 * t0] = b->surfTri[k] - H.v0;
  if (detect_now) {
    launch_begin_step(b->d, b->stream);
    launch_collisions(b->d, b->d.coll, b->stream);
    CUDA_TRY(cudaGetLastError());
  }
  std::vector<int> offs(s1 - s0 + 1), cand((size_t)kMaxPairsPerVertex * (s1 - s0));
  CUDA_TRY(cudaMemcpyAsync(offs.data(), b->d.coll.svCount + s0, sizeof(int) * offs.size(), cudaMemcpyDeviceToHost,
                           b->stream));
  CUDA_TRY(cudaMemcpyAsync(cand.data(), b->d.coll.svCand + (size_t)kMaxPairsPerVertex * s0,
                           sizeof(int) * cand.size(), cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  int n = 0;
  for (int i = 0; i < s1 - s0; i++) {
    const int c = offs[i + 1] - offs[i];
    for (int j = 0; j < c; j++, n++)
      if (pairs && n < cap) {
        pairs[2 * n] = b->svHost[s0 + i] - H.v0;
        pairs[2 * n + 1] = cand[(size_t)kMaxPairsPerVertex * i + j] - t0;
      }
  }
  if (npairs) *npairs = n;
  return HOBAK_OK;
}

int hobak_batch_collision_response(hobak_batch b, int scene, int cap, int* tets, double* force, double* hessian) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (!b->collArena) return fail(HOBAK_ERR_INVALID, "collisions were never enabled on this batch");
  const SceneHost& H = b->scenes[scene];
  const int s0 = b->svStart[scene], s1 = b->svStart[scene + 1];
  int p0 = 0, p1 = 0;
  CUDA_TRY(cudaMemcpy(&p0, b->d.coll.svCount + s0, sizeof(int), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(&p1, b->d.coll.svCount + s1, sizeof(int), cudaMemcpyDeviceToHost));
  const int n = std::min(p1 - p0, cap);
  if (n <= 0) return HOBAK_OK;
  std::vector<int4> ct(n);
  std::vector<double> C(4 * (size_t)n), G(9 * (size_t)n), F(12 * (size_t)n);
  CUDA_TRY(cudaMemcpy(ct.data(), b->d.coll.pairTet + p0, sizeof(int4) * n, cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(C.data(), b->d.coll.pairC + 4 * (size_t)p0, sizeof(double) * C.size(), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(G.data(), b->d.coll.pairG + 9 * (size_t)p0, sizeof(double) * G.size(), cudaMemcpyDeviceToHost));
  CUDA_TRY(cudaMemcpy(F.data(), b->d.coll.pairF + 12 * (size_t)p0, sizeof(double) * F.size(), cudaMemcpyDeviceToHost));
  for (int k = 0; k < n; k++) {
    if (tets) {
      tets[4 * k] = ct[k].x - H.v0;
      tets[4 * k + 1] = ct[k].y - H.v0;
      tets[4 * k + 2] = ct[k].z - H.v0;
      tets[4 * k + 3] = ct[k].w - H.v0;
    }
    if (force) std::copy(&F[12 * (size_t)k], &F[12 * (size_t)k + 12], force + 12 * (size_t)k);
    if (hessian)
      for (int a = 0; a < 4; a++)
        for (int bb = 0; bb < 4; bb++)
          for (int i = 0; i < 3; i++)
            for (int j = 0; j < 3; j++)
              hessian[144 * (size_t)k + (3 * a + i) + 12 * (3 * bb + j)] =
                  C[4 * (size_t)k + a] * C[4 * (size_t)k + bb] * G[9 * (size_t)k + i + 3 * j];
  }
  return HOBAK_OK;
}

int hobak_batch_set_active(hobak_batch b, int scene, int active) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  b->sceneParams[scene].active = active ? 1 : 0;
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(b->d.scenes) + scene, &b->sceneParams[scene], sizeof(SceneParams),
                      cudaMemcpyHostToDevice));
  if (b->collArena) {  // a parked scene takes no part in collision detection either
    CollisionScene cs = b->collScenes[scene];
    if (!active) cs.vfOn = cs.eeOn = 0;
    CUDA_TRY(cudaMemcpy(const_cast<CollisionScene*>(b->d.coll.scenes) + scene, &cs, sizeof(CollisionScene),
                        cudaMemcpyHostToDevice));
  }
  return HOBAK_OK;
}

int hobak_batch_device_bytes(hobak_batch b, long long* bytes) {
  if (!b || !bytes) return fail(HOBAK_ERR_INVALID, "bad arguments");
  *bytes = (long long)(b->arenaBytes + b->precBytes + (b->K0 ? sizeof(double) * 9 * (size_t)b->nblocks : 0));
  return HOBAK_OK;
}

int hobak_batch_energy(hobak_batch b, int scene, double* energy) {
  if (!b || !energy || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const SceneHost& H = b->scenes[scene];
  launch_energy(b->d, b->stream);
  std::vector<double> psi(H.nt);
  CUDA_TRY(cudaMemcpyAsync(psi.data(), b->d.psi + H.t0, sizeof(double) * H.nt, cudaMemcpyDeviceToHost, b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  double e = 0;
  for (double p : psi) e += p;
  *energy = e;
  return HOBAK_OK;
}

int hobak_batch_get_stream(hobak_batch b, void** stream) {
  if (!b || !stream) return fail(HOBAK_ERR_INVALID, "bad arguments");
  *stream = (void*)b->stream;
  return HOBAK_OK;
}

int hobak_batch_enable_timing(hobak_batch b, int on) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  b->timing = on != 0;
  return HOBAK_OK;
}

int hobak_batch_phase_times(hobak_batch b, double* ms, long long* launches) {
  if (!b) return fail(HOBAK_ERR_INVALID, "null handle");
  for (int k = 0; k < 5; k++) {
    if (ms) ms[k] = b->phaseMs[k];
    if (launches) launches[k] = b->phaseLaunches[k];
    b->phaseMs[k] = 0;
    b->phaseLaunches[k] = 0;
  }
  return HOBAK_OK;
}

int hobak_batch_launch_count(hobak_batch b, long long* launches) {
  if (!b || !launches) return fail(HOBAK_ERR_INVALID, "bad arguments");
  long long loop = 0;
  int rc = count_loop_launches(b, &loop);
  if (rc) return rc;
  *launches = b->launches + loop;
  return HOBAK_OK;
}

int hobak_batch_time_kernels(hobak_batch b, int reps, double* ms) {
  if (!b || !ms || reps <= 0) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const DeviceBatch& d = b->d;
  cudaStream_t s = b->stream;
  const int n = (int)b->scenes.size();
  cudaEvent_t e0 = b->ev[0], e1 = b->ev[1];
  const bool mixed = b->opts.precision == HOBAK_PRECISION_MIXED;
  // the PCG loop kernels run over every tile of every scene (also the scenes
  // a cluster solves in the step: this times the tile-path kernels over the
  // whole batch) from a real inner-solve start, and keep every scene's PCG
  // running so that each launch does its full work (a negative inner
  // threshold also leaves the scalars alone: repeated SpMVs on the same
  // vectors would drive the recurrences to infinity)
  auto keep_running = [&]() -> int {
    std::vector<SolveState> st(n);
    CUDA_TRY(cudaMemcpy(st.data(), d.solve, sizeof(SolveState) * n, cudaMemcpyDeviceToHost));
    for (auto& x : st) {
      x.done = 0;
      x.outerDone = 0;
      x.newtonDone = 0;
      x.innerThreshold = -1.0;
      x.maxit = 0x7fffffff;
      x.totalIters = 0;
    }
    CUDA_TRY(cudaMemcpy(d.solve, st.data(), sizeof(SolveState) * n, cudaMemcpyHostToDevice));
    return HOBAK_OK;
  };
  if (int rc = keep_running()) return rc;  // (Newmark: no scene counts as finished)
  for (int k = 0; k < 4; k++) {
    if (k == 2) {
      std::vector<SceneParams> sp = b->sceneParams;
      for (auto& x : sp) x.pcgCluster = 0;
      CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(d.scenes), sp.data(), sizeof(SceneParams) * n,
                          cudaMemcpyHostToDevice));
      if (int rc = keep_running()) return rc;
      if (mixed) launch_inner_init<float>(d, d.v32, s);
      else launch_inner_init<double>(d, d.v64, s);
      CUDA_TRY(cudaStreamSynchronize(s));
      if (int rc = keep_running()) return rc;
      CUDA_TRY(cudaMemcpyAsync(d.nLoopTiles, &d.ntiles, sizeof(int), cudaMemcpyHostToDevice, s));
    }
    CUDA_TRY(cudaEventRecord(e0, s));
    for (int r = 0; r < reps; r++) {
      if (k == 0) {
        if (mixed) launch_element_mixed(d, s);
        else launch_element(d, s);
      } else if (k == 1) {
        if (mixed) launch_assemble<float>(d, d.v32, s);
        else launch_assemble<double>(d, d.v64, s);
      } else if (k == 2) {
        if (mixed) launch_spmv<float>(d, d.v32, s);
        else launch_spmv<double>(d, d.v64, s);
      } else {
        if (mixed) launch_update<float>(d, d.v32, s);
        else launch_update<double>(d, d.v64, s);
      }
    }
    CUDA_TRY(cudaEventRecord(e1, s));
    CUDA_TRY(cudaEventSynchronize(e1));
    float t = 0;
    CUDA_TRY(cudaEventElapsedTime(&t, e0, e1));
    ms[k] = t / reps;
  }
  b->launches += (3LL + element_launches(d, mixed)) * reps + 1;
  CUDA_TRY(cudaGetLastError());
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(d.scenes), b->sceneParams.data(), sizeof(SceneParams) * n,
                      cudaMemcpyHostToDevice));
  return upload_solver_opts(b);
}

int hobak_batch_get_tuning(hobak_batch b, hobak_tuning* out) {
  if (!b || !out) return fail(HOBAK_ERR_INVALID, "bad arguments");
  out->tile_vertices = b->d.tileV;
  out->element_threads = b->d.elemThreads;
  out->assembly_threads = b->d.asmThreads;
  out->pcg_chunk = b->chunk;
  out->cluster_pcg = b->clusterPcg ? 1 : 0;
  out->cluster_max = b->clusterMax;
  out->step_ms = 0.0;
  return HOBAK_OK;
}

int hobak_batch_set_green_damping(hobak_batch b, int scene, double mu) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (b->opts.integrator != HOBAK_INTEGRATOR_NEWMARK)
    return fail(HOBAK_ERR_INVALID, "GREEN_DAMPING: only NEWMARK's energy-damped solve is defined");
  if (!(mu >= 0.0) || !std::isfinite(mu)) return fail(HOBAK_ERR_INVALID, "damping mu must be finite and >= 0");
  b->sceneParams[scene].greenMu = mu;
  int any = 0;
  for (const SceneParams& p : b->sceneParams) any |= p.greenMu > 0.0 ? 1 : 0;
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  CUDA_TRY(cudaMemcpy(const_cast<SceneParams*>(b->d.scenes) + scene, &b->sceneParams[scene], sizeof(SceneParams),
                      cudaMemcpyHostToDevice));
  if (any != b->d.anyGreen) {  // the Newton body gains or loses a kernel
    b->d.anyGreen = any;
    drop_graphs(b);
  }
  return HOBAK_OK;
}

int hobak_batch_set_scene_cluster(hobak_batch b, int scene, int ctas) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  if (!(ctas == -1 || ctas == 0 || ctas == 1 || ctas == 2 || ctas == 4 || ctas == 8 || ctas == 16))
    return fail(HOBAK_ERR_INVALID, "ctas must be -1 (tile path), 0 (by the tuning), 1, 2, 4, 8 or 16");
  if (b->sceneCluster.size() != b->scenes.size()) b->sceneCluster.assign(b->scenes.size(), 0);
  if (b->sceneCluster[scene] != ctas) {
    b->sceneCluster[scene] = ctas;
    b->clusterDirty = true;
  }
  return HOBAK_OK;
}

int hobak_batch_pcg_path(hobak_batch b, int* cluster_ctas) {
  if (!b || !cluster_ctas) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (int rc = prepare_cluster_classes(b)) return rc;
  for (size_t s = 0; s < b->scenes.size(); s++) cluster_ctas[s] = b->sceneParams[s].pcgCluster;
  return HOBAK_OK;
}

int hobak_batch_set_tuning(hobak_batch b, const hobak_tuning* t) {
  if (!b || !t) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (t->element_threads != 64 && t->element_threads != 128)
    return fail(HOBAK_ERR_INVALID, "element_threads must be 64 or 128");
  if (t->assembly_threads < 64 || t->assembly_threads > 1024 || t->assembly_threads % 32 != 0)
    return fail(HOBAK_ERR_INVALID, "assembly_threads must be a multiple of 32 in 64..1024");
  if (t->pcg_chunk < 1 || t->pcg_chunk > 64) return fail(HOBAK_ERR_INVALID, "pcg_chunk must be in 1..64");
  if (t->tile_vertices != 64 && t->tile_vertices != 128)
    return fail(HOBAK_ERR_INVALID, "tile_vertices must be 64 or 128");
  if (t->cluster_pcg != 0 && t->cluster_pcg != 1) return fail(HOBAK_ERR_INVALID, "cluster_pcg must be 0 or 1");
  if (t->cluster_max != 1 && t->cluster_max != 2 && t->cluster_max != 4 && t->cluster_max != 8 && t->cluster_max != 16)
    return fail(HOBAK_ERR_INVALID, "cluster_max must be 1, 2, 4, 8 or 16");
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  if (t->tile_vertices != b->d.tileV) {
    const int rc = apply_tile_size(b, t->tile_vertices);
    if (rc) return rc;
  }
  if (t->pcg_chunk != b->chunk) {
    const int rc = fold_loop_launches(b);
    if (rc) return rc;
    b->chunk = t->pcg_chunk;
  }
  b->d.elemThreads = t->element_threads;
  b->d.asmThreads = t->assembly_threads;
  if ((t->cluster_pcg != 0) != b->clusterPcg || t->cluster_max != b->clusterMax) {
    b->clusterPcg = t->cluster_pcg != 0;
    b->clusterMax = t->cluster_max;
    b->clusterDirty = true;
  }
  drop_graphs(b);
  return HOBAK_OK;
}

namespace {
struct DeviceScratch {
  void* p = nullptr;
  ~DeviceScratch() {
    if (p) cudaFree(p);
  }
};
struct EventPair {
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  ~EventPair() {
    if (e0) cudaEventDestroy(e0);
    if (e1) cudaEventDestroy(e1);
  }
};
}  // namespace

int hobak_batch_autotune(hobak_batch b, int reps, hobak_tuning* out) {
  if (!b || reps <= 0) return fail(HOBAK_ERR_INVALID, "bad arguments");
  DeviceBatch& d = b->d;
  cudaStream_t s = b->stream;
  const bool mixed = b->opts.precision == HOBAK_PRECISION_MIXED;
  const size_t vbytes = 3 * sizeof(double) * (size_t)b->nv;
  CUDA_TRY(cudaStreamSynchronize(s));
  DeviceScratch saved;
  CUDA_TRY(cudaMalloc(&saved.p, 3 * vbytes));
  double* x0 = static_cast<double*>(saved.p);
  double* v0 = x0 + 3 * (size_t)b->nv;
  double* a0 = v0 + 3 * (size_t)b->nv;  // Newmark's acceleration
  CUDA_TRY(cudaMemcpyAsync(x0, d.x, vbytes, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(v0, d.v, vbytes, cudaMemcpyDeviceToDevice, s));
  CUDA_TRY(cudaMemcpyAsync(a0, d.acc, vbytes, cudaMemcpyDeviceToDevice, s));
  auto restore = [&]() -> int {
    CUDA_TRY(cudaMemcpyAsync(d.x, x0, vbytes, cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.v, v0, vbytes, cudaMemcpyDeviceToDevice, s));
    CUDA_TRY(cudaMemcpyAsync(d.acc, a0, vbytes, cudaMemcpyDeviceToDevice, s));
    return HOBAK_OK;
  };
  EventPair ev;
  CUDA_TRY(cudaEventCreate(&ev.e0));
  CUDA_TRY(cudaEventCreate(&ev.e1));
  auto elapsed = [&](float* ms) -> int {
    CUDA_TRY(cudaEventSynchronize(ev.e1));
    CUDA_TRY(cudaEventElapsedTime(ms, ev.e0, ev.e1));
    return HOBAK_OK;
  };
  hobak_tuning best{};
  hobak_batch_get_tuning(b, &best);
  // 1. element kernel CTA size (inputs are the saved state; outputs are
  //    recomputed by every step)
  {
    float bestMs = 3.4e38f;
    for (int et : {64, 128}) {
      d.elemThreads = et;
      CUDA_TRY(cudaEventRecord(ev.e0, s));
      for (int r = 0; r < reps; r++) {
        if (mixed) launch_element_mixed(d, s);
        else launch_element(d, s);
      }
      CUDA_TRY(cudaEventRecord(ev.e1, s));
      float ms = 0;
      int rc = elapsed(&ms);
      if (rc) return rc;
      b->launches += (long long)reps * element_launches(d, mixed);
      if (ms < bestMs) {
        bestMs = ms;
        best.element_threads = et;
      }
    }
    d.elemThreads = best.element_threads;
  }
  // 2. assembly kernel CTA size
  {
    float bestMs = 3.4e38f;
    for (int at : {64, 128, 256, 512}) {
      d.asmThreads = at;
      // one untimed launch first: the candidates are timed warm alike
      if (mixed) launch_assemble<float>(d, d.v32, s);
      else launch_assemble<double>(d, d.v64, s);
      b->launches += 1;
      CUDA_TRY(cudaEventRecord(ev.e0, s));
      for (int r = 0; r < reps; r++) {
        if (mixed) launch_assemble<float>(d, d.v32, s);
        else launch_assemble<double>(d, d.v64, s);
      }
      CUDA_TRY(cudaEventRecord(ev.e1, s));
      float ms = 0;
      int rc = elapsed(&ms);
      if (rc) return rc;
      b->launches += reps;
      if (ms < bestMs) {
        bestMs = ms;
        best.assembly_threads = at;
      }
    }
    d.asmThreads = best.assembly_threads;
  }
  // 3. whole steps per (PCG path: tile path only, or clusters of at most 4,
  //    8 or 16 CTAs for the scenes that fit; tile size; chunk), each from the
  //    saved state
  double bestStep = 1e300;
  hobak_tuning trial = best;
  const int paths[4][2] = {{0, 16}, {1, 4}, {1, 8}, {1, 16}};
  for (const auto& path : paths)
  for (int tv : {64, 128})
    for (int ch : {4, 8, 16}) {
      trial.cluster_pcg = path[0];
      trial.cluster_max = path[1];
      trial.tile_vertices = tv;
      trial.pcg_chunk = ch;
      int rc = hobak_batch_set_tuning(b, &trial);
      if (rc) return rc;
      if ((rc = restore())) return rc;
      if ((rc = run_steps(b, 1))) return rc;  // builds this shape's graph
      double total = 0.0;
      for (int r = 0; r < reps; r++) {
        if ((rc = restore())) return rc;
        CUDA_TRY(cudaEventRecord(ev.e0, s));
        if ((rc = run_steps(b, 1))) return rc;
        CUDA_TRY(cudaEventRecord(ev.e1, s));
        float ms = 0;
        if ((rc = elapsed(&ms))) return rc;
        total += ms;
      }
      if (total < bestStep) {
        bestStep = total;
        best.cluster_pcg = path[0];
        best.cluster_max = path[1];
        best.tile_vertices = tv;
        best.pcg_chunk = ch;
      }
    }
  best.step_ms = bestStep / reps;
  int rc = hobak_batch_set_tuning(b, &best);
  if (rc) return rc;
  if ((rc = restore())) return rc;
  CUDA_TRY(cudaStreamSynchronize(s));
  if ((rc = upload_solver_opts(b))) return rc;
  if (out) *out = best;
  return HOBAK_OK;
}

int hobak_batch_kernel_bytes(hobak_batch b, double* bytes) {
  if (!b || !bytes) return fail(HOBAK_ERR_INVALID, "bad arguments");
  const double T = b->nt, V = b->nv, B = b->nblocks, C = 16.0 * b->nt;
  const double w = b->opts.precision == HOBAK_PRECISION_MIXED ? 4.0 : 8.0;  // inner value width
  // element: tets 16, 4 x (rest, x, v) 288, DmInv 72, vol 8, scene id 4; writes 90 Hessian values + 12 doubles
  bytes[0] = T * (16 + 288 + 72 + 8 + 4 + w * kElemHess + 96);
  // assembly: element Hessians once, contribution map, block row/col/ptr, LHS write; mask/mass/scene per vertex
  bytes[1] = T * w * kElemHess + C * 4 + B * (4 + 4 + 4 + 9 * w) + V * (1 + 8 + 4);
  // spmv: LHS row block + column per block; rowptr, u read and w written per vertex
  bytes[2] = B * (9 * w + 4) + V * (4 + 2 * 3 * w);
  // update: u, p rw, w, s rw, d rw, r rw, Minv (9), u write per vertex
  bytes[3] = V * w * (3 + 6 + 3 + 6 + 6 + 6 + 9 + 3);
  return HOBAK_OK;
}

int hobak_gpu_create(const hobak_scene_desc* scene, const hobak_solver_opts* opts, hobak_batch* out) {
  return hobak_batch_create(scene, 1, opts, out);
}
int hobak_gpu_step(hobak_batch b, int nsteps, hobak_step_stats* stats) { return hobak_batch_step(b, nsteps, stats); }
int hobak_gpu_set_state(hobak_batch b, const double* x, const double* v) { return hobak_batch_set_state(b, 0, x, v); }
int hobak_gpu_get_state(hobak_batch b, double* x, double* v) { return hobak_batch_get_state(b, 0, x, v); }
int hobak_gpu_set_external_forces(hobak_batch b, const double* f) { return hobak_batch_set_external_forces(b, 0, f); }
int hobak_gpu_set_collisions(hobak_batch b, int vf_on, double eps, double stiffness, double damping_beta) {
  return hobak_batch_set_collisions(b, 0, vf_on, eps, stiffness, damping_beta);
}
int hobak_gpu_set_edge_collisions(hobak_batch b, int ee_on) { return hobak_batch_set_edge_collisions(b, 0, ee_on); }
int hobak_gpu_set_solver(hobak_batch b, const hobak_solver_opts* opts) { return hobak_batch_set_solver(b, opts); }
int hobak_gpu_destroy(hobak_batch b) { return hobak_batch_destroy(b); }

namespace {
// psi / PK1 / clampedHessian / hessian of n elements given F, or (U, Sigma, V)
// when U is not null; one device allocation for inputs and outputs.
int material_eval(const hobak_material* m, int n, const double* F, const double* U, const double* S,
                  const double* V, double* psi, double* P, double* H, double* Hu) {
  if (!m || n <= 0 || (!F && !(U && S && V))) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (int rc = validate_material(*m, 0)) return rc;
  int rc = hobak_device_check(nullptr, nullptr, nullptr);
  if (rc) return rc;
  const size_t N = (size_t)n;
  // inputs (F: 9, or U, Sigma, V: 21) then outputs psi 1, P 9, H 81, Hu 81 per element
  const size_t nin = U ? 21 : 9;
  const size_t nout = (psi ? 1 : 0) + (P ? 9 : 0) + (H ? 81 : 0) + (Hu ? 81 : 0);
  DeviceScratch scratch;
  CUDA_TRY(cudaMalloc(&scratch.p, (nin + nout) * N * sizeof(double)));
  double* cur = static_cast<double*>(scratch.p);
  auto take = [&](size_t per) {
    double* p = cur;
    cur += per * N;
    return p;
  };
  double *dF = nullptr, *dU = nullptr, *dS = nullptr, *dV = nullptr;
  if (U) {
    dU = take(9);
    dS = take(3);
    dV = take(9);
    CUDA_TRY(cudaMemcpy(dU, U, 9 * N * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dS, S, 3 * N * sizeof(double), cudaMemcpyHostToDevice));
    CUDA_TRY(cudaMemcpy(dV, V, 9 * N * sizeof(double), cudaMemcpyHostToDevice));
  } else {
    dF = take(9);
    CUDA_TRY(cudaMemcpy(dF, F, 9 * N * sizeof(double), cudaMemcpyHostToDevice));
  }
  double* dPsi = psi ? take(1) : nullptr;
  double* dP = P ? take(9) : nullptr;
  double* dH = H ? take(81) : nullptr;
  double* dHu = Hu ? take(81) : nullptr;
  launch_material_eval(m->kind, m->mu, m->lambda, m->fiber, n, dF, dU, dS, dV, dPsi, dP, dH, dHu, 0);
  CUDA_TRY(cudaGetLastError());
  if (psi) CUDA_TRY(cudaMemcpy(psi, dPsi, N * sizeof(double), cudaMemcpyDeviceToHost));
  if (P) CUDA_TRY(cudaMemcpy(P, dP, 9 * N * sizeof(double), cudaMemcpyDeviceToHost));
  if (H) CUDA_TRY(cudaMemcpy(H, dH, 81 * N * sizeof(double), cudaMemcpyDeviceToHost));
  if (Hu) CUDA_TRY(cudaMemcpy(Hu, dHu, 81 * N * sizeof(double), cudaMemcpyDeviceToHost));
  return HOBAK_OK;
}
}  // namespace

int hobak_material_eval(const hobak_material* m, int n, const double* F, double* psi, double* P, double* H) {
  if (!F) return fail(HOBAK_ERR_INVALID, "bad arguments");
  return material_eval(m, n, F, nullptr, nullptr, nullptr, psi, P, H, nullptr);
}

int hobak_material_hessian(const hobak_material* m, int n, const double* F, double* H) {
  if (!F || !H) return fail(HOBAK_ERR_INVALID, "bad arguments");
  return material_eval(m, n, F, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, H);
}

int hobak_material_eval_svd(const hobak_material* m, int n, const double* U, const double* sigma, const double* V,
                            double* psi, double* P, double* H, double* clampedH) {
  if (!U || !sigma || !V) return fail(HOBAK_ERR_INVALID, "bad arguments");
  return material_eval(m, n, nullptr, U, sigma, V, psi, P, clampedH, H);
}

int hobak_material_needs_svd(int kind, int* energy, int* pk1) {
  if (kind < HOBAK_MATERIAL_SNH || kind > HOBAK_MATERIAL_ANISOTROPIC_DIRICHLET)
    return fail(HOBAK_ERR_INVALID, "unknown material");
  // energyNeedsSVD / PK1NeedsSVD as each material class answers them
  // (SNH.cpp, ARAP.cpp, STVK.cpp, LINEAR.cpp, NEO_HOOKEAN_BW.cpp,
  // SNH_WITH_BARRIER.cpp, ANISOTROPIC_*.cpp)
  static const int e[10] = {0, 1, 0, 0, 0, 0, 1, 1, 1, 0};
  static const int p[10] = {0, 1, 0, 0, 0, 0, 1, 1, 1, 0};
  if (energy) *energy = e[kind];
  if (pk1) *pk1 = p[kind];
  return HOBAK_OK;
}

int hobak_element_eval(int nv, int nt, const double* rest, const int* tets, const double* x, const hobak_material* m,
                       double* F, double* sigma, double* force, double* hessian) {
  if (nv <= 0 || nt <= 0 || !rest || !tets || !x || !m) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (int rc = validate_material(*m, 0)) return rc;
  for (long k = 0; k < 4L * nt; k++)
    if (tets[k] < 0 || tets[k] >= nv) return fail(HOBAK_ERR_INVALID, "tet vertex id out of range");
  int rc = hobak_device_check(nullptr, nullptr, nullptr);
  if (rc) return rc;
  std::vector<double> Dm(9 * (size_t)nt), vol(nt);
  for (int t = 0; t < nt; t++) {
    const double* p[4];
    for (int a = 0; a < 4; a++) p[a] = rest + 3 * (size_t)tets[4 * (size_t)t + a];
    vol[t] = tet_volume(p[0], p[1], p[2], p[3]);
    dm_inverse(p[0], p[1], p[2], p[3], &Dm[9 * (size_t)t]);
  }
  const size_t T = (size_t)nt, V = (size_t)nv;
  double *dRest, *dX, *dDm, *dVol, *dF = nullptr, *dS = nullptr, *dFo = nullptr, *dH = nullptr;
  int4* dTets;
  CUDA_TRY(cudaMalloc(&dRest, 3 * V * sizeof(double)));
  CUDA_TRY(cudaMalloc(&dX, 3 * V * sizeof(double)));
  CUDA_TRY(cudaMalloc(&dDm, 9 * T * sizeof(double)));
  CUDA_TRY(cudaMalloc(&dVol, T * sizeof(double)));
  CUDA_TRY(cudaMalloc(&dTets, T * sizeof(int4)));
  if (F) CUDA_TRY(cudaMalloc(&dF, 9 * T * sizeof(double)));
  if (sigma) CUDA_TRY(cudaMalloc(&dS, 3 * T * sizeof(double)));
  if (force) CUDA_TRY(cudaMalloc(&dFo, 12 * T * sizeof(double)));
  if (hessian) CUDA_TRY(cudaMalloc(&dH, 144 * T * sizeof(double)));
  CUDA_TRY(cudaMemcpy(dRest, rest, 3 * V * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(dX, x, 3 * V * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(dDm, Dm.data(), 9 * T * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(dVol, vol.data(), T * sizeof(double), cudaMemcpyHostToDevice));
  CUDA_TRY(cudaMemcpy(dTets, tets, T * sizeof(int4), cudaMemcpyHostToDevice));
  launch_element_eval(nt, dTets, dRest, dX, dDm, dVol, m->kind, m->mu, m->lambda, m->fiber, dF, dS, dFo, dH, 0);
  CUDA_TRY(cudaGetLastError());
  if (F) CUDA_TRY(cudaMemcpy(F, dF, 9 * T * sizeof(double), cudaMemcpyDeviceToHost));
  if (sigma) CUDA_TRY(cudaMemcpy(sigma, dS, 3 * T * sizeof(double), cudaMemcpyDeviceToHost));
  if (force) CUDA_TRY(cudaMemcpy(force, dFo, 12 * T * sizeof(double), cudaMemcpyDeviceToHost));
  if (hessian) CUDA_TRY(cudaMemcpy(hessian, dH, 144 * T * sizeof(double), cudaMemcpyDeviceToHost));
  for (void* p : {(void*)dRest, (void*)dX, (void*)dDm, (void*)dVol, (void*)dTets, (void*)dF, (void*)dS,
                  (void*)dFo, (void*)dH})
    cudaFree(p);
  return HOBAK_OK;
}

int hobak_batch_assemble(hobak_batch b, int scene, int* nblocks, int* rowptr, int* cols, double* K, double* R) {
  if (!b || scene < 0 || scene >= (int)b->scenes.size()) return fail(HOBAK_ERR_INVALID, "bad handle or scene");
  const SceneHost& H = b->scenes[scene];
  const int rb0 = b->hostRowptr[H.v0], rb1 = b->hostRowptr[H.v0 + H.nv];
  if (nblocks) *nblocks = rb1 - rb0;
  if (rowptr)
    for (int u = 0; u <= H.nv; u++) rowptr[u] = b->hostRowptr[H.v0 + u] - rb0;
  if (cols)
    for (int k = rb0; k < rb1; k++) cols[k - rb0] = b->hostCols[k] - H.v0;
  if (!K && !R) return HOBAK_OK;
  // element terms at the current state with raw forces (FP64 element
  // Hessians in scratch of this call), then the device gathers K (CSR
  // order, scratch) and R (into the per-step rhs buffer)
  DeviceScratch scratch;
  const size_t ehBytes = sizeof(double) * kElemHessStride * (size_t)b->nt;
  CUDA_TRY(cudaMalloc(&scratch.p, ehBytes + sizeof(double) * 9 * (size_t)std::max(b->nblocks, 1)));
  DeviceBatch d = b->d;
  d.elemH = static_cast<double*>(scratch.p);
  double* Kd = reinterpret_cast<double*>(static_cast<char*>(scratch.p) + ehBytes);
  launch_begin_step(d, b->stream);
  launch_element(d, b->stream, 1);
  launch_assemble_raw(d, Kd, d.rhs, b->stream);
  CUDA_TRY(cudaGetLastError());
  if (K)
    CUDA_TRY(cudaMemcpyAsync(K, Kd + 9 * (size_t)rb0, 9 * sizeof(double) * (rb1 - rb0), cudaMemcpyDeviceToHost,
                             b->stream));
  if (R)
    CUDA_TRY(cudaMemcpyAsync(R, d.rhs + 3 * (size_t)H.v0, 3 * sizeof(double) * H.nv, cudaMemcpyDeviceToHost,
                             b->stream));
  CUDA_TRY(cudaStreamSynchronize(b->stream));
  return HOBAK_OK;
}

}  // extern "C"
