// Cluster-resident PCG for small scenes.
//
// One thread-block cluster solves one scene's linear system from start to
// finish in a single launch: the scene's vertices are split into CL
// contiguous ranges, one per CTA; the Krylov vectors of a range live in that
// CTA's shared memory, the SpMV gathers the search vector of neighbouring
// ranges from the other CTAs' shared memory (distributed shared memory), and
// every dot product is a CTA tree followed by a fixed-order sum of the CL CTA
// partials read through distributed shared memory.  An iteration is two
// cluster barriers (the fused reduction after the SpMV, and the publication
// of the new u after the update); the matrix and Minv are read from L2 (or
// DRAM, when a full batch's other scenes have evicted them) every iteration.
// In mixed precision the launch also runs every refinement sweep: the FP64
// y update, the residual update r -= A d in compensated FP32 and the outer
// FP64 test, then the next inner solve, until the test passes.  A scene in
// contact adds its rows' contact terms from the step's pair lists.  The tile
// path (solver.cu: two grid-wide kernels per iteration, each ending in a
// ticketed reduction) remains for scenes too large for a cluster.
//
// The iteration is the same Chronopoulos-Gear PCG as the tile path, with the
// same scalars, stopping rules and iteration accounting (ConjugateGradient.h
// stopping rule; the FP64 path's verdict from the recursive residual), so the
// two paths agree to rounding.  Thread 0 of every CTA computes the scalars
// from the same partials in the same order, hence every CTA takes the same
// branches and reaches every barrier.
#include <cooperative_groups.h>

#include <atomic>
#include <cfloat>

#include "kernels.cuh"

namespace cg = cooperative_groups;

namespace hobak {

namespace {

__device__ __forceinline__ bool finite_d(double x) { return x == x && fabs(x) <= DBL_MAX; }

// Shared memory of one CTA:
//   [slots: 8 doubles][warp partials: 3 * kClusterWarps doubles][ubase: 16 u32]
//   [u: 4 * vpc T (x, y, z, 0 per vertex: one vector load per gather)]
//   [p, s, w, d, r: 3 * vpc T each]
constexpr int kSlotBytes = 8 * sizeof(double) + 3 * kClusterWarps * sizeof(double) + 16 * sizeof(uint32_t);

template <typename T>
struct ClusterSmem {
  double* slots;     // [1..3] the loop's reductions, [4..6] the initial one (cluster_sum3)
  T* warp;           // 3 * kClusterWarps warp partials
  uint32_t* ubase;   // shared::cluster address of u in every CTA of the cluster
  T *u, *p, *s, *w, *d, *r;
};

template <typename T>
__device__ __forceinline__ ClusterSmem<T> carve_smem(unsigned char* base, int vpc) {
  ClusterSmem<T> m;
  m.slots = reinterpret_cast<double*>(base);
  m.warp = reinterpret_cast<T*>(base + 8 * sizeof(double));
  m.ubase = reinterpret_cast<uint32_t*>(base + 8 * sizeof(double) + 3 * kClusterWarps * sizeof(double));
  T* v = reinterpret_cast<T*>(base + kSlotBytes);
  const int n = 3 * vpc;
  m.u = v;
  m.p = v + 4 * vpc;
  m.s = m.p + n;
  m.w = m.s + n;
  m.d = m.w + n;
  m.r = m.d + n;
  return m;
}

// The u of a vertex in any CTA of the cluster, by its shared::cluster address
// (mapa of the owner's u plus the local offset): one vector load.
__device__ __forceinline__ void ld_u(uint32_t a, float* x) {
  float pad;
  asm volatile("ld.shared::cluster.v4.f32 {%0, %1, %2, %3}, [%4];"
               : "=f"(x[0]), "=f"(x[1]), "=f"(x[2]), "=f"(pad)
               : "r"(a));
}
__device__ __forceinline__ void ld_u(uint32_t a, double* x) {
  double pad;
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x[0]), "=d"(x[1]) : "r"(a));
  asm volatile("ld.shared::cluster.v2.f64 {%0, %1}, [%2];" : "=d"(x[2]), "=d"(pad) : "r"(a + 16));
}
__device__ __forceinline__ uint32_t map_cluster(const void* p, int rank) {
  uint32_t out;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;"
               : "=r"(out)
               : "r"((uint32_t)__cvta_generic_to_shared(p)), "r"(rank));
  return out;
}
__device__ __forceinline__ double ld_cluster_f64(uint32_t a) {
  double x;
  asm volatile("ld.shared::cluster.f64 %0, [%1];" : "=d"(x) : "r"(a));
  return x;
}

// The contact rows of vertex u of w H_coll x (w = collision_lhs_scale of the
// scene; H_coll = the sum over u's collision tets of (c c^T) (x) G, as
// collision_row on the tile path), with x read four wide from the cluster's
// shared memory: the scene's vertex id - v0 lies in the range of CTA
// (id - v0) / vpc.  FP64 sums of the FP32 x (the contact blocks are not part
// of the FP32 LHS).  Only free rows carry contact (pinned x are zero).
// The per-step contact arrays contact_rows reads (DeviceCollisions).
struct ContactRefs {
  const int* incCount;
  const int* incList;
  const int4* pairTet;
  const double* pairC;
  const double* pairG;
};

template <typename T>
__device__ __forceinline__ void contact_rows(const ContactRefs& c, int u, int v0, int vpc, double scale,
                                             const uint32_t* ubase, double out[3]) {
  constexpr int kUShift = sizeof(T) == 4 ? 4 : 5;
  out[0] = out[1] = out[2] = 0.0;
  const int k0 = c.incCount[u], k1 = c.incCount[u + 1];
  for (int k = k0; k < k1; k++) {
    const int e = c.incList[k], p = e >> 2, a = e & 3;
    const int4 ct = c.pairTet[p];
    const double* C = c.pairC + 4 * (size_t)p;
    const double* G = c.pairG + 9 * (size_t)p;
    const int id[4] = {ct.x, ct.y, ct.z, ct.w};
    double z[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < 4; q++) {
      const int w = id[q] - v0, owner = w / vpc;
      T x[3];
      ld_u(ubase[owner] + ((uint32_t)(w - owner * vpc) << kUShift), x);
#pragma unroll
      for (int j = 0; j < 3; j++) z[j] += C[q] * double(x[j]);
    }
#pragma unroll
    for (int i = 0; i < 3; i++) out[i] += C[a] * (G[i] * z[0] + G[i + 3] * z[1] + G[i + 6] * z[2]);
  }
#pragma unroll
  for (int i = 0; i < 3; i++) out[i] *= scale;
}

// Three sums over the cluster: a warp tree, the CTA's warps summed by a tree
// in warp 0 (in T, widened to FP64 once), a cluster barrier, then lanes
// 0..CL-1 of warp 0 read the CL CTA sums through distributed shared memory
// and a warp tree adds them.  Every tree is fixed, so results are
// reproducible and independent of other scenes.  The sums are valid in warp 0
// of every CTA (all its lanes).  The scalar recurrences that follow run in one
// thread per CTA: 1024 threads redoing FP64 divisions would occupy GB300's
// 2-lane FP64 pipe for tens of microseconds per iteration.
// slot: the first of the three slots the CTA sums go to.  The loop's
// reductions use slots 1..3 (the previous one's remote reads end before the
// cluster barrier that closes its iteration); the initial one uses 4..6, so
// no CTA overwrites a slot another may not have read yet.
template <int CL, typename T>
__device__ __forceinline__ void cluster_sum3(cg::cluster_group& cluster, const ClusterSmem<T>& m, T a, T b, T c,
                                             int slot, double (&out)[3]) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int wid = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) {
    m.warp[3 * wid] = a;
    m.warp[3 * wid + 1] = b;
    m.warp[3 * wid + 2] = c;
  }
  __syncthreads();
  if (wid == 0) {
    T ta = m.warp[3 * lane], tb = m.warp[3 * lane + 1], tc = m.warp[3 * lane + 2];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      ta += __shfl_xor_sync(0xffffffffu, ta, o);
      tb += __shfl_xor_sync(0xffffffffu, tb, o);
      tc += __shfl_xor_sync(0xffffffffu, tc, o);
    }
    if (lane == 0) {
      m.slots[slot] = double(ta);
      m.slots[slot + 1] = double(tb);
      m.slots[slot + 2] = double(tc);
    }
  }
  cluster.sync();
  out[0] = out[1] = out[2] = 0.0;
  if (wid == 0) {
    double sa = 0.0, sb = 0.0, sc = 0.0;
    if (lane < CL) {
      const uint32_t sl = map_cluster(m.slots + slot, lane);
      sa = ld_cluster_f64(sl);
      sb = ld_cluster_f64(sl + 8);
      sc = ld_cluster_f64(sl + 16);
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      sa += __shfl_xor_sync(0xffffffffu, sa, o);
      sb += __shfl_xor_sync(0xffffffffu, sb, o);
      sc += __shfl_xor_sync(0xffffffffu, sc, o);
    }
    out[0] = sa;
    out[1] = sb;
    out[2] = sc;
  }
}

// One FP64 sum over the cluster (the residual's |r64|^2): the same trees as
// cluster_sum3, on FP64 warp partials.  Valid in warp 0 of every CTA.
template <int CL, typename T>
__device__ __forceinline__ double cluster_sum_f64(cg::cluster_group& cluster, const ClusterSmem<T>& m, double a,
                                                  int slot) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(0xffffffffu, a, o);
  double* warp = reinterpret_cast<double*>(m.warp);  // sized for 3 doubles per warp
  const int wid = threadIdx.x / 32, lane = threadIdx.x % 32;
  if (lane == 0) warp[wid] = a;
  __syncthreads();
  if (wid == 0) {
    double t = lane < kClusterWarps ? warp[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) m.slots[slot] = t;
  }
  cluster.sync();
  double out = 0.0;
  if (wid == 0) {
    double sa = lane < CL ? ld_cluster_f64(map_cluster(m.slots + slot, lane)) : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sa += __shfl_xor_sync(0xffffffffu, sa, o);
    out = sa;
  }
  return out;
}

// a * x + (s, c): the exact product (TwoProduct: rounded product and its
// error by an FMA) added to the running sum s with the addition's error
// (TwoSum) and the product's error gathered in c.  Rounded operations only
// (__fmul_rn / __fadd_rn are never contracted), so the error terms are exact.
__device__ __forceinline__ void dot2_step(float a, float x, float& s, float& c) {
  const float p = __fmul_rn(a, x);
  const float pe = __fmaf_rn(a, x, -p);
  const float t = __fadd_rn(s, p);
  const float bp = __fsub_rn(t, s);
  const float se = __fadd_rn(__fsub_rn(s, __fsub_rn(t, bp)), __fsub_rn(p, bp));
  s = t;
  c = __fadd_rn(c, __fadd_rn(se, pe));
}

// The end of a mixed-precision sweep for vertices [u0, u0 + n) of a scene.
// y += rsc d in FP64; the correction d is published four wide in u's place
// (u is rebuilt by the next sweep's start); a cluster barrier (release /
// acquire); then the residual is updated, r64 -= rsc (A d), with A d formed
// from the FP32 blocks and the FP32 d by compensated dot products (Dot2 of
// Ogita, Rump and Oishi: as accurate as FP64 sums of the exact products, on
// the FP32 pipes rather than GB300's 2-lane FP64 pipe), and |r64|^2 summed
// over the cluster (valid in warp 0).  r64 starts as rhs (y = 0), so it is
// rhs - A y up to FP64 rounding of the updates.  Not inlined: its registers
// stay out of the PCG loop's allocation.
template <int CL>
__device__ __noinline__ double sweep_residual(cg::cluster_group& cluster, const ClusterSmem<float>& m, double* y,
                                              double* r64, const int* gather, const int* sliceRow, const int* rowptr,
                                              const float* lhs, int u0, int n, double rsc,
                                              bool contact, ContactRefs coll, const unsigned char* freeMask,
                                              int v0, int vpc, double collScale) {
  for (int lv = threadIdx.x; lv < n; lv += kClusterThreads) {
    const int u = u0 + lv;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float di = m.d[3 * lv + i];
      y[3 * u + i] += rsc * double(di);
      m.u[4 * lv + i] = di;
    }
    m.u[4 * lv + 3] = 0.0f;
  }
  cluster.sync();
  double rl = 0.0;
  for (int lv = threadIdx.x; lv < n; lv += kClusterThreads) {
    const int u = u0 + lv;
    const int len = rowptr[u + 1] - rowptr[u];
    const size_t srow = (size_t)sliceRow[u >> 5];
    const float* B = lhs + srow * kSlotVals + (u & (kSlice - 1));
    const int* G = gather + srow * kSlice + (u & (kSlice - 1));
    float s[3] = {0.0f, 0.0f, 0.0f}, c[3] = {0.0f, 0.0f, 0.0f};
    for (int j = 0; j < len; j++) {
      const int g = __ldg(G + j * kSlice);
      float x[3];
      ld_u(m.ubase[g >> 20] + ((uint32_t)(g & 0xFFFFF) << 4), x);
      const float* Bj = B + (size_t)kSlotVals * j;
#pragma unroll
      for (int i = 0; i < 3; i++)
#pragma unroll
        for (int k = 0; k < 3; k++) dot2_step(Bj[(3 * i + k) * kSlice], x[k], s[i], c[i]);
    }
    double cr[3] = {0.0, 0.0, 0.0};
    if (contact && freeMask[u]) contact_rows<float>(coll, u, v0, vpc, collScale, m.ubase, cr);
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double ri = r64[3 * u + i] - rsc * (double(s[i]) + double(c[i]) + cr[i]);
      r64[3 * u + i] = ri;
      rl += ri * ri;
    }
  }
  return cluster_sum_f64<CL>(cluster, m, rl, 7);
}
template <int CL>
__device__ double sweep_residual(cg::cluster_group&, const ClusterSmem<double>&, double*, double*, const int*,
                                 const int*, const int*, const double*, int, int, double, bool, ContactRefs,
                                 const unsigned char*, int, int, double) {
  return 0.0;  // FP64: one inner solve is the solve; never called
}

// The scene's PCG and sweep scalars, kept by thread 0 of each CTA.
struct Scalars {
  double innerThr = 0.0, gamma = 0.0, gammaOld = 1.0, alpha = 1.0, beta = 0.0, srr = 0.0;
  int maxit = 0, totalIters = 0, iters = 0, converged = 0, outerDone = 0, sweep = 0;
};

// Values thread 0 hands to the CTA after each reduction.
template <typename T>
struct Broadcast {
  double scale;  // mixed: the next sweep's residual scale
  T alpha, beta;
  int stop;      // 1: the inner solve (or the sweeps) ended; 2: non-finite, the step failed
};

// Owner CTA and local vertex index of every slot's column for the scenes
// solved in clusters (gather[slot] = owner << 20 | local index; the owner is
// the CTA whose range [owner * vpc, (owner + 1) * vpc) holds the column), in
// the sliced layout of colS.  Built when the cluster assignment changes.
__global__ void k_cluster_gather(DeviceBatch b, int* __restrict__ gather) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)b.nslotRows * kSlice) return;
  const int u = b.slotSlice[i / kSlice] * kSlice + (int)(i % kSlice);
  int g = 0;
  if (u < b.nv) {
    const SceneParams& sp = b.scenes[b.vertexScene[u]];
    if (sp.pcgCluster > 0) {
      const int vpc = (sp.nv + sp.pcgCluster - 1) / sp.pcgCluster;
      const int w = b.colS[i] - sp.v0;
      const int owner = w / vpc;
      g = (owner << 20) | (w - owner * vpc);
    }
  }
  gather[i] = g;
}

template <int CL, typename T>
__global__ void __cluster_dims__(CL, 1, 1) __launch_bounds__(kClusterThreads, 1)
    k_pcg_cluster(DeviceBatch b, PcgVecs<T> v, const int* __restrict__ sceneList,
                  const int* __restrict__ gather) {
  cg::cluster_group cluster = cg::this_cluster();
  const int rank = (int)cluster.block_rank();
  const int sc = sceneList[blockIdx.x / CL];
  SolveState& st = b.solve[sc];
  const SceneParams& sp = b.scenes[sc];
  const bool t0 = threadIdx.x == 0;
  const bool lead = rank == 0 && t0;
  // a finished or parked scene: nothing to solve (same for every CTA)
  if (st.outerDone) {
    if (lead) st.done = 1;
    return;
  }
  extern __shared__ __align__(16) unsigned char smem[];
  __shared__ Broadcast<T> bc;
  const int v0 = sp.v0, nvS = sp.nv;
  const int vpc = (nvS + CL - 1) / CL;  // the scene's own split: alone == in any batch
  const ClusterSmem<T> m = carve_smem<T>(smem, vpc);
  const int my0 = min(nvS, rank * vpc), my1 = min(nvS, (rank + 1) * vpc);
  const int nmine = my1 - my0;
  // contact on this scene: its rows add w H_coll u (collision_lhs_scale)
  const bool contact = b.collOn && (b.coll.scenes[sc].vfOn || b.coll.scenes[sc].eeOn);
  constexpr int kUShift = sizeof(T) == 4 ? 4 : 5;  // bytes of one u entry: 16 (float4) or 32
  if (threadIdx.x < CL) m.ubase[threadIdx.x] = map_cluster(m.u, threadIdx.x);

  // The scene's scalar state, kept by thread 0 of every CTA in shared memory
  // (identical copies, computed from the same cluster sums in the same
  // order); registers stay with the SpMV.
  __shared__ Scalars ss;
  if (t0) {
    ss = Scalars{};
    ss.maxit = st.maxit;
    ss.totalIters = st.totalIters;
    ss.converged = st.converged;
    ss.sweep = st.sweep;
    // mixed: the power-of-two scale of this sweep's r
    bc.scale = (sizeof(T) != sizeof(double) && st.rScale > 0.0) ? st.rScale : 1.0;
  }
  __syncthreads();
  // Mixed precision: every refinement sweep runs here, back to back (the
  // scene's own y, FP64 residual and outer test, as k_accumulate and
  // k_residual do for the tile path), so a scene's sweeps never wait for
  // the rest of the batch.
  double sums[3];
  for (;;) {
    // ---- init: r = r64 / rsc (the FP64 residual, scaled and rounded), u = Minv r, d = p = s = 0 ----
    const double rsc = bc.scale;
    const double inv = 1.0 / rsc;  // exact: rsc is a power of two
    T rr = T(0), ru = T(0);
    for (int lv = threadIdx.x; lv < nmine; lv += kClusterThreads) {
      const int u = v0 + my0 + lv;
      T r3[3];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        r3[i] = T(b.r64[3 * u + i] * inv);
        m.r[3 * lv + i] = r3[i];
        m.d[3 * lv + i] = T(0);
        m.p[3 * lv + i] = T(0);
        m.s[3 * lv + i] = T(0);
        rr += r3[i] * r3[i];
      }
      const T* M = v.minv + 9 * (size_t)u;
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const T ui = M[3 * i] * r3[0] + M[3 * i + 1] * r3[1] + M[3 * i + 2] * r3[2];
        m.u[4 * lv + i] = ui;
        ru += r3[i] * ui;
      }
      m.u[4 * lv + 3] = T(0);
    }
    cluster_sum3<CL, T>(cluster, m, rr, ru, T(0), 4, sums);
    if (t0) {
      ss.srr = sums[0];
      double itol = st.tol;
      if (sizeof(T) != sizeof(double))
        itol = fmax(st.tol * sqrt(st.rhsNorm2 / fmax(ss.srr * rsc * rsc, DBL_MIN)), st.innerFloor);
      ss.innerThr = fmax(itol * itol * ss.srr, DBL_MIN);
      ss.gamma = sums[1];
      ss.gammaOld = 1.0;
      ss.alpha = 1.0;
      ss.beta = 0.0;
      ss.iters = 0;
      bc.stop = (ss.srr == 0.0 || ss.srr < ss.innerThr) ? 1 : 0;
    }
    __syncthreads();
    while (!bc.stop) {
      // ---- w = A u over my vertices; delta = (w, u), gamma = (r, u), |r|^2 ----
      T dl = T(0), gl = T(0), rl = T(0);
      for (int lv = threadIdx.x; lv < nmine; lv += kClusterThreads) {
        const int u = v0 + my0 + lv;
        T a0 = T(0), a1 = T(0), a2 = T(0);
        const int len = b.rowptr[u + 1] - b.rowptr[u];
        const size_t srow = (size_t)b.sliceRow[u >> 5];
        // the row's sliced 3x3 blocks (entry e of block j at (j * 288 + 32 e))
        // and gather entries (j * 32), four blocks per trip with the next
        // trip's gather entries fetched one trip ahead
        const T* B = v.lhs + srow * kSlotVals + (u & (kSlice - 1));
        const int* G = gather + srow * kSlice + (u & (kSlice - 1));
        int gn[4];
  #pragma unroll
        for (int q = 0; q < 4; q++) gn[q] = q < len ? __ldg(G + q * kSlice) : 0;
        for (int j = 0; j < len; j += 4) {
          int gq[4];
  #pragma unroll
          for (int q = 0; q < 4; q++) {
            gq[q] = gn[q];
            gn[q] = (j + 4 + q < len) ? __ldg(G + (j + 4 + q) * kSlice) : 0;
          }
          T x[4][3];
  #pragma unroll
          for (int q = 0; q < 4; q++) {
            const uint32_t a = m.ubase[gq[q] >> 20] + ((uint32_t)(gq[q] & 0xFFFFF) << kUShift);
            ld_u(a, x[q]);
          }
  #pragma unroll
          for (int q = 0; q < 4; q++) {
            if (j + q < len) {
              const T* Bq = B + (size_t)kSlotVals * (j + q);
              a0 = fma(Bq[0], x[q][0], fma(Bq[kSlice], x[q][1], fma(Bq[2 * kSlice], x[q][2], a0)));
              a1 = fma(Bq[3 * kSlice], x[q][0], fma(Bq[4 * kSlice], x[q][1], fma(Bq[5 * kSlice], x[q][2], a1)));
              a2 = fma(Bq[6 * kSlice], x[q][0], fma(Bq[7 * kSlice], x[q][1], fma(Bq[8 * kSlice], x[q][2], a2)));
            }
          }
        }
        if (contact && b.freeMask[u]) {
          const ContactRefs coll{b.coll.incCount, b.coll.incList, b.coll.pairTet, b.coll.pairC, b.coll.pairG};
          double cr[3];
          contact_rows<T>(coll, u, v0, vpc, collision_lhs_scale(b, sc), m.ubase, cr);
          a0 += T(cr[0]);
          a1 += T(cr[1]);
          a2 += T(cr[2]);
        }
        m.w[3 * lv] = a0;
        m.w[3 * lv + 1] = a1;
        m.w[3 * lv + 2] = a2;
        const T u0 = m.u[4 * lv], u1 = m.u[4 * lv + 1], u2 = m.u[4 * lv + 2];
        const T r0 = m.r[3 * lv], r1 = m.r[3 * lv + 1], r2 = m.r[3 * lv + 2];
        dl += a0 * u0 + a1 * u1 + a2 * u2;
        gl += r0 * u0 + r1 * u1 + r2 * u2;
        rl += r0 * r0 + r1 * r1 + r2 * r2;
      }
      cluster_sum3<CL, T>(cluster, m, rl, gl, dl, 1, sums);
      if (t0) {
        // after an update: the convergence test on its residual, then the
        // scalars of this iteration's update (tile path: spmv_decide)
        int stop = 0;
        if (ss.iters > 0) {
          ss.srr = sums[0];
          if (ss.srr < ss.innerThr) {
            stop = 1;
          } else if (!finite_d(ss.srr) || !finite_d(sums[1]) || !finite_d(ss.alpha)) {
            stop = 2;  // the step fails: no further sweep
            ss.converged = -1;
            ss.outerDone = 1;
          } else if (ss.totalIters >= ss.maxit) {
            stop = 1;
          }
        }
        if (!stop) {
          const double g = sums[1], delta = sums[2];
          if (ss.iters == 0) {
            ss.beta = 0.0;
            ss.alpha = g / delta;
          } else {
            ss.beta = g / ss.gamma;
            ss.alpha = g / (delta - ss.beta * g / ss.alpha);
          }
          ss.gammaOld = ss.gamma;
          ss.gamma = g;
          ss.iters += 1;
          ss.totalIters += 1;
        }
        bc.alpha = T(ss.alpha);
        bc.beta = T(ss.beta);
        bc.stop = stop;
      }
      __syncthreads();
      if (bc.stop) break;
      const T ta = bc.alpha, tb = bc.beta;
      // ---- p = u + beta p, s = w + beta s, d += alpha p, r -= alpha s, u = Minv r ----
      for (int lv = threadIdx.x; lv < nmine; lv += kClusterThreads) {
        const int u = v0 + my0 + lv;
        T r3[3];
  #pragma unroll
        for (int i = 0; i < 3; i++) {
          const int j = 3 * lv + i;
          const T p = m.u[4 * lv + i] + tb * m.p[j];
          const T sv = m.w[j] + tb * m.s[j];
          m.p[j] = p;
          m.s[j] = sv;
          m.d[j] += ta * p;
          r3[i] = m.r[j] - ta * sv;
          m.r[j] = r3[i];
        }
        const T* M = v.minv + 9 * (size_t)u;
  #pragma unroll
        for (int i = 0; i < 3; i++) m.u[4 * lv + i] = M[3 * i] * r3[0] + M[3 * i + 1] * r3[1] + M[3 * i + 2] * r3[2];
      }
      // the new u reaches the other CTAs' SpMV
      cluster.sync();
    }
    if (sizeof(T) == sizeof(double)) break;  // FP64: the inner solve is the solve
    if (bc.stop == 2) break;                 // non-finite: the step has failed
    // ---- mixed: y += rsc d, r64 -= rsc A d, |r64|^2 ----
    const double s64 = sweep_residual<CL>(cluster, m, b.y, b.r64, gather, b.sliceRow, b.rowptr, v.lhs, v0 + my0,
                                          nmine, rsc, contact,
                                          ContactRefs{b.coll.incCount, b.coll.incList, b.coll.pairTet, b.coll.pairC,
                                                      b.coll.pairG},
                                          b.freeMask, v0, vpc, contact ? collision_lhs_scale(b, sc) : 0.0);
    if (t0) {
      // the outer test (tile path: k_residual)
      ss.sweep += 1;
      int done = 0;
      if (s64 < st.threshold) {
        done = 1;
        ss.converged = 1;
      } else if (!finite_d(s64)) {
        done = 1;
        ss.converged = -1;
      } else if (ss.sweep >= st.maxSweeps || ss.totalIters >= ss.maxit) {
        done = 1;
        ss.converged = 0;
      }
      ss.outerDone = done;
      ss.srr = s64;
      bc.scale = pow2_near_norm(s64);
      bc.stop = done;
    }
    __syncthreads();
    if (bc.stop) break;
  }
  // ---- results: FP64 path, the solution y itself (the correction d) ----
  if (sizeof(T) == sizeof(double)) {
    for (int lv = threadIdx.x; lv < nmine; lv += kClusterThreads) {
      const int u = v0 + my0 + lv;
#pragma unroll
      for (int i = 0; i < 3; i++) v.d[3 * u + i] = m.d[3 * lv + i];
    }
  }
  if (lead) {
    st.rr = ss.srr;
    st.iters = ss.iters;
    st.totalIters = ss.totalIters;
    st.gamma = ss.gamma;
    st.gammaOld = ss.gammaOld;
    st.alpha = ss.alpha;
    st.beta = ss.beta;
    st.innerThreshold = ss.innerThr;
    st.done = 1;
    if (sizeof(T) == sizeof(double)) {
      if (ss.outerDone) {
        st.converged = ss.converged;
      } else {
        // FP64 path: the recursive residual is the solver's verdict (Eigen)
        st.rr64 = ss.srr;
        st.converged = ss.srr < st.threshold ? 1 : 0;
      }
    } else {
      st.sweep = ss.sweep;
      st.rr64 = ss.srr;
      st.rScale = bc.scale;
      st.converged = ss.converged;
    }
    st.outerDone = 1;
  }
  // no CTA leaves while another may still read its shared memory
  cluster.sync();
}

template <int CL, typename T>
int launch_class(const DeviceBatch& b, const PcgVecs<T>& v, const ClusterClass& c, cudaStream_t s) {
  if (c.count == 0) return 0;
  const size_t smem = kSlotBytes + cluster_vertex_bytes(sizeof(T) == 4) * c.vpcMax;
  k_pcg_cluster<CL, T><<<c.count * CL, kClusterThreads, smem, s>>>(b, v, c.scenes, b.clusterGather);
  return 0;
}

template <int CL, typename T>
cudaError_t allow_smem() {
  cudaError_t e = cudaFuncSetAttribute(k_pcg_cluster<CL, T>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       (int)kClusterSmemMax);
  if (e == cudaSuccess && CL > 8)  // 16-CTA clusters are a non-portable size
    e = cudaFuncSetAttribute(k_pcg_cluster<CL, T>, cudaFuncAttributeNonPortableClusterSizeAllowed, 1);
  return e;
}

}  // namespace

// Opt every cluster kernel into kClusterSmemMax bytes of dynamic shared
// memory (once per process; outside any stream capture; batches may be
// created and stepped from several host threads).
int configure_cluster_pcg() {
  static std::atomic<int> done{0};
  if (done.load()) return 0;
  cudaError_t e = cudaSuccess;
  if (e == cudaSuccess) e = allow_smem<1, float>();
  if (e == cudaSuccess) e = allow_smem<2, float>();
  if (e == cudaSuccess) e = allow_smem<4, float>();
  if (e == cudaSuccess) e = allow_smem<8, float>();
  if (e == cudaSuccess) e = allow_smem<16, float>();
  if (e == cudaSuccess) e = allow_smem<1, double>();
  if (e == cudaSuccess) e = allow_smem<2, double>();
  if (e == cudaSuccess) e = allow_smem<4, double>();
  if (e == cudaSuccess) e = allow_smem<8, double>();
  if (e == cudaSuccess) e = allow_smem<16, double>();
  if (e != cudaSuccess) return (int)e;
  done.store(1);
  return 0;
}

// u (4 wide) and p, s, w, d, r (3 wide) per vertex
size_t cluster_vertex_bytes(bool mixed) { return (size_t)19 * (mixed ? sizeof(float) : sizeof(double)); }

void launch_cluster_gather(const DeviceBatch& b, cudaStream_t s) {
  const size_t n = (size_t)b.nslotRows * kSlice;
  if (n == 0) return;
  k_cluster_gather<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, b.clusterGather);
}
size_t cluster_fixed_bytes() { return kSlotBytes; }

template <typename T>
int launch_cluster_pcg(const DeviceBatch& b, const PcgVecs<T>& v, const ClusterClass* classes, int k, cudaStream_t s) {
  switch (k) {
    case 0: return launch_class<1, T>(b, v, classes[0], s);
    case 1: return launch_class<2, T>(b, v, classes[1], s);
    case 2: return launch_class<4, T>(b, v, classes[2], s);
    case 3: return launch_class<8, T>(b, v, classes[3], s);
    default: return launch_class<16, T>(b, v, classes[4], s);
  }
}
template int launch_cluster_pcg<double>(const DeviceBatch&, const PcgVecs<double>&, const ClusterClass*, int,
                                        cudaStream_t);
template int launch_cluster_pcg<float>(const DeviceBatch&, const PcgVecs<float>&, const ClusterClass*, int,
                                       cudaStream_t);

}  // namespace hobak
