// Assembly, right-hand side, PCG and refinement kernels.
//
// System of one BACKWARD_EULER_VELOCITY step (BACKWARD_EULER_VELOCITY.cpp:157-176):
//   b   = dt (R + dt K v + f_ext)
//   A   = M - dt^2 K                      (C = 0: TIMESTEPPER.cpp:657)
//   LHS = S A S + (I - S),  rhs = S b     (S = 0 blocks at pinned vertices)
// solved from y = 0 with the stopping rule of Eigen's conjugate_gradient
// (ConjugateGradient.h:28-90): |r|^2 < max(tol^2 |rhs|^2, DBL_MIN) on the
// recursive residual.
//
// PCG runs in the Chronopoulos-Gear arrangement (same iterates as the
// textbook loop in exact arithmetic) with its three dot products fused into
// one reduction, so each iteration is two kernels and a single scene-wide
// reduction, and the SpMV multiplies a vector that is already final:
//   k_spmv:   w = A u; delta = (w, u), gamma = (r, u), |r|^2
//             -> convergence test on |r|^2 (the residual of the last
//                update), then beta, alpha
//   k_update: p = u + beta p, s = w + beta s, d += alpha p, r -= alpha s,
//             u = Minv r  (no reduction)
// The test on |r_k|^2 thus runs at the start of iteration k rather than at
// the end of k - 1: same decision, same iterates and iteration count; a
// stopping scene computes one SpMV it does not use.
// On GB300 the FP64 pipe, not HBM, bounds the FP64 SpMV, so the product does
// only the 9 DFMA per block it must (one thread per vertex, no lane
// reductions).  The LHS is stored in 32-vertex slices (lhs_slot), so the
// SpMV's matrix and column loads are whole 128-byte lines per warp.
//
// Mixed precision: the inner PCG runs on FP32 vectors and an FP32 matrix; the
// outer loop keeps y and the residual rhs - A y in FP64 (iterative refinement,
// at most 1 + max_refinements sweeps) and stops on the same FP64 test.
//
// No atomics touch values: every matrix block and vertex sums its element
// contributions in ascending tet order, and every dot product is a fixed tree
// (per-tile partials, then the last tile of the scene sums them in tile
// order), so results are bitwise reproducible and a scene's result does not
// depend on the batch around it.
#include <algorithm>
#include <cfloat>

#include "kernels.cuh"

namespace hobak {

namespace {

// Tile kernels are instantiated for every supported tile size TV (vertices
// per tile): vector kernels and the SpMV run one thread per vertex (TV
// threads), the update and residual one thread per scalar row.  The batch's
// tile size is an autotuned launch shape (DeviceBatch::tileV).

// Fixed-order sum over the CTA; result valid in thread 0.  NT multiple of 32.
// The whole tree runs in R (FP32 for the inner solve of the mixed path) and
// only the CTA's total is widened to FP64: a conversion per warp costs a
// 16-cycle issue on GB300's 2-lane FP64 pipe even when one lane uses it.
template <int NT, typename R>
__device__ __forceinline__ double block_sum(R v, double* sh) {
  R* shr = reinterpret_cast<R*>(sh);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) shr[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0) {
    R t = R(0);
#pragma unroll
    for (int i = 0; i < NT / 32; i++) t += shr[i];
    s = double(t);
  }
  __syncthreads();
  return s;
}

// Two sums in one pass (one pair of barriers); results valid in thread 0.
// `sh` holds 2 * NT / 32 doubles.
template <int NT, typename R>
__device__ __forceinline__ void block_sum2(R a, R b, double* sh, double& sa, double& sb) {
  R* shr = reinterpret_cast<R*>(sh);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
  }
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) {
    shr[w] = a;
    shr[NT / 32 + w] = b;
  }
  __syncthreads();
  sa = 0.0;
  sb = 0.0;
  if (threadIdx.x == 0) {
    R ta = R(0), tb = R(0);
#pragma unroll
    for (int i = 0; i < NT / 32; i++) {
      ta += shr[i];
      tb += shr[NT / 32 + i];
    }
    sa = double(ta);
    sb = double(tb);
  }
  __syncthreads();
}

// Three sums in one pass (one pair of barriers), each in the order of
// block_sum; results valid in thread 0.  `sh` holds 3 * NT / 32 doubles.
template <int NT, typename R>
__device__ __forceinline__ void block_sum3(R a, R b, R c, double* sh, double (&out)[3]) {
  R* shr = reinterpret_cast<R*>(sh);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    a += __shfl_xor_sync(0xffffffffu, a, o);
    b += __shfl_xor_sync(0xffffffffu, b, o);
    c += __shfl_xor_sync(0xffffffffu, c, o);
  }
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) {
    shr[w] = a;
    shr[NT / 32 + w] = b;
    shr[2 * (NT / 32) + w] = c;
  }
  __syncthreads();
  out[0] = out[1] = out[2] = 0.0;
  if (threadIdx.x == 0) {
    R ta = R(0), tb = R(0), tc = R(0);
#pragma unroll
    for (int i = 0; i < NT / 32; i++) {
      ta += shr[i];
      tb += shr[NT / 32 + i];
      tc += shr[2 * (NT / 32) + i];
    }
    out[0] = double(ta);
    out[1] = double(tb);
    out[2] = double(tc);
  }
  __syncthreads();
}

// After thread 0 wrote the CTA's partial(s): true in the CTA that finishes
// the scene's reduction (ticket == ntiles - 1).  Only thread 0 published
// anything the last CTA reads, so only it fences before taking its ticket.
// The ticket is reset for reuse.
__device__ __forceinline__ bool last_tile(unsigned* ticket, int ntiles, int* flag) {
  if (threadIdx.x == 0) {
    __threadfence();
    const unsigned t = atomicAdd(ticket, 1u);
    *flag = (t == (unsigned)(ntiles - 1));
    if (*flag) *ticket = 0u;
  }
  __syncthreads();
  const bool last = *flag != 0;
  if (last) __threadfence();
  return last;
}

// Sum partial[(tile0 + i) * kPartials + comp] over i < n in a fixed order.
template <int NT>
__device__ __forceinline__ double sum_partials(const double* partial, int tile0, int n, int comp, double* sh) {
  double s = 0;
  for (int i = threadIdx.x; i < n; i += NT) s += __ldcg(&partial[(size_t)(tile0 + i) * kPartials + comp]);
  return block_sum<NT>(s, sh);
}

// Partials 0..2 of a scene's tiles, each summed in tile order (one pass).
template <int NT>
__device__ __forceinline__ void sum_partials3(const double* partial, int tile0, int n, double* sh, double (&out)[3]) {
  double a = 0, b = 0, c = 0;
  for (int i = threadIdx.x; i < n; i += NT) {
    const double* q = partial + (size_t)(tile0 + i) * kPartials;
    a += __ldcg(q);
    b += __ldcg(q + 1);
    c += __ldcg(q + 2);
  }
  block_sum3<NT>(a, b, c, sh, out);
}

__device__ __forceinline__ bool finite(double x) { return x == x && fabs(x) <= DBL_MAX; }

// Programmatic dependent launch (sm_90 and later).  The PCG loop kernels are
// launched with programmatic stream serialisation: the next kernel's CTAs may
// start once every CTA of the running one has called pdl_trigger (or exited),
// do the loads that do not depend on it (tile tables, matrix rows, column
// indices, Minv rows: all written before the loop), and pdl_wait before
// touching anything it writes (vectors, partials, solve state).  Every CTA
// triggers at its start, so all CTAs of a kernel are resident or finished
// before any CTA of the next one waits: no CTA can wait on one that cannot
// run.  Launched without the attribute, pdl_wait returns at once.
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// The update kernel puts 10 vertices (30 scalar rows) in each warp so that a
// vertex's three rows share a warp: ceil(TV / 10) warps per tile.
__host__ __device__ constexpr int update_warps(int TV) { return (TV + 9) / 10; }

// x[pinned] = pin target at the start of a step
// (applyKinematicConstraints, TIMESTEPPER.cpp:105-122).
// Newmark also keeps the step's starting x, v, a (before the pins move x).
__global__ void k_begin_step(DeviceBatch b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv) return;
  if (b.scenes[b.vertexScene[u]].integrator == kIntegratorNewmark)
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const size_t q = 3 * (size_t)u + i;
      b.xOld[q] = b.x[q];
      b.vOld[q] = b.v[q];
      b.aOld[q] = b.acc[q];
    }
  if (b.freeMask[u]) return;
#pragma unroll
  for (int i = 0; i < 3; i++) b.x[3 * u + i] = b.pinTarget[3 * u + i];
}

// Newmark: every active scene starts its Newton loop (one CTA over scenes);
// other integrators and parked scenes count as finished.
__global__ void __launch_bounds__(256) k_newton_begin(DeviceBatch b) {
  __shared__ int total;
  if (threadIdx.x == 0) total = 0;
  __syncthreads();
  int n = 0;
  for (int s = threadIdx.x; s < b.nscenes; s += blockDim.x) {
    SolveState& st = b.solve[s];
    const bool run = b.scenes[s].active && b.scenes[s].integrator == kIntegratorNewmark;
    st.newtonStep = 0;
    st.newtonDone = run ? 0 : 1;
    n += run ? 1 : 0;
  }
  atomicAdd(&total, n);
  __syncthreads();
  if (threadIdx.x == 0) *b.newtonActive = total;
}

// Newmark, after a solve: x -= y for the scenes still iterating.
__global__ void k_newton_step(DeviceBatch b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv || b.solve[b.vertexScene[u]].newtonDone) return;
#pragma unroll
  for (int i = 0; i < 3; i++) b.x[3 * u + i] -= b.y[3 * u + i];
}

// ... then each scene's Newton test: stop once the iteration just done
// started from |rhs|^2 <= eps, or after maxNewton iterations
// (NEWMARK.cpp:216: while step < max && maxR > eps).
__global__ void __launch_bounds__(256) k_newton_test(DeviceBatch b) {
  int finished = 0;
  for (int s = threadIdx.x; s < b.nscenes; s += blockDim.x) {
    SolveState& st = b.solve[s];
    if (st.newtonDone) continue;
    st.newtonStep += 1;
    const SceneParams& sp = b.scenes[s];
    if (!(st.newtonR > sp.newtonEps) || st.newtonStep >= sp.maxNewton) {
      st.newtonDone = 1;
      finished++;
    }
  }
  if (finished) atomicSub(b.newtonActive, finished);
}

// Graph loop control of the Newton loop.
__global__ void k_newton_continue(const int* newtonActive, unsigned long long* runs, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *runs += 1ull;
    cudaGraphSetConditional(h, *newtonActive > 0 ? 1u : 0u);
  }
}

// Sum of one block entry over its element contributions, ascending tet
// (TET_MESH_FASTER.cpp:113-131 gathers the same entries per non-zero).
// The sum is formed in HT: FP64 for the FP64 path, FP32 for the mixed path
// (whose matrix is FP32 anyway; converting every term would load the FP64 pipe).
// Contributions are fetched eight at a time (all map entries, then all
// values, as independent loads) and added in list order, so a diagonal block
// with ~24 incident tets waits on 6 memory latencies instead of 48.
template <typename HT>
__device__ __forceinline__ HT gather_block_entry(const DeviceBatch& b, const HT* __restrict__ elemH, int blk,
                                                 int r, int c) {
  HT sum = HT(0);
  const int k1 = b.blkptr[blk + 1];
  for (int k = b.blkptr[blk]; k < k1; k += 8) {
    int src[8];
#pragma unroll
    for (int q = 0; q < 8; q++) src[q] = (k + q < k1) ? __ldg(&b.blksrc[k + q]) : 0;
    HT val[8];
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int t = src[q] >> 4, ea = (src[q] >> 2) & 3, eb = src[q] & 3;
      const HT* H = elemH + (size_t)kElemHessStride * t;
      val[q] = (k + q >= k1) ? HT(0)
               : (ea <= eb)  ? H[9 * upper_block(ea, eb) + 3 * r + c]
                             : H[9 * upper_block(eb, ea) + 3 * c + r];
    }
#pragma unroll
    for (int q = 0; q < 8; q++)
      if (k + q < k1) sum += val[q];
  }
  return sum;
}

// Slot of the sliced LHS -> CSR block: slot row r, lane -> vertex u, block
// k = rowptr[u] + j; false for padding slots and lanes past the last vertex.
__device__ __forceinline__ bool slot_block(const DeviceBatch& b, int r, int lane, int& u, int& k) {
  const int sl = b.slotSlice[r];
  u = kSlice * sl + lane;
  if (u >= b.nv) return false;
  const int j = r - b.sliceRow[sl];
  const int k0 = b.rowptr[u];
  if (j >= b.rowptr[u + 1] - k0) return false;
  k = k0 + j;
  return true;
}

// FP64 assembly: one thread per (slot, entry), entries of a slot on nine
// neighbouring lanes, so the nine entries of a contribution (72 contiguous
// bytes) are read in one request; at FP64 width this coalescing beats a
// thread per block.
template <typename HT, typename T>
__global__ void k_assemble_entry(DeviceBatch b, const HT* __restrict__ elemH, T* __restrict__ lhs) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (size_t)kSlotVals * b.nslotRows) return;
  const int r = (int)(g / kSlotVals), rem = (int)(g % kSlotVals);
  const int lane = rem / 9, e = rem % 9;
  int u, blk;
  if (!slot_block(b, r, lane, u, blk)) return;
  if (!b.scenes[b.vertexScene[u]].active || b.solve[b.vertexScene[u]].newtonDone) return;
  const int rr = e / 3, c = e % 3;
  const HT sum = gather_block_entry(b, elemH, blk, rr, c);
  const int w = b.cols[blk];
  const SceneParams& sp = b.scenes[b.vertexScene[u]];
  const double dt = sp.dt;
  const bool fu = b.freeMask[u] != 0, fw = b.freeMask[w] != 0;
  HT val;
  if (sp.integrator == kIntegratorPosition) {
    // A = M (1/dt^2 - alpha/dt) - (beta/dt) K0 - K (BACKWARD_EULER_POSITION.cpp:207)
    const double invDt = 1.0 / dt;
    val = (fu && fw) ? HT(-(sp.rayBeta * invDt)) * HT(b.K0[9 * (size_t)blk + rr + 3 * c]) - sum : HT(0);
    if (u == w && rr == c) val += fu ? HT(b.mass[u] * (invDt * invDt - sp.rayAlpha * invDt)) : HT(1);
  } else if (sp.integrator == kIntegratorNewmark) {
    // A = alpha_0 M - K (NEWMARK.cpp:262; its C is zeroed before use)
    val = (fu && fw) ? -sum : HT(0);
    if (u == w && rr == c) val += fu ? HT(sp.nm[0] * b.mass[u]) : HT(1);
  } else {
    val = (fu && fw) ? HT(-(dt * dt)) * sum : HT(0);
    if (u == w && rr == c) val += fu ? HT(b.mass[u]) : HT(1);
  }
  lhs[(size_t)r * kSlotVals + kSlice * e + lane] = T(val);
}

// FP32 assembly: one thread per slot (a warp per slot row of 32 vertices):
// the block's 9 entries summed over its element contributions in list order
// (ascending tet), several contributions' loads in flight at a time (each
// contribution is 9 contiguous values: a 3x3 block of one element Hessian,
// transposed for the lower triangle), then LHS block = S(M - dt^2 K)S + (I - S)
// written entry by entry, each entry of the warp's 32 slots one 128-byte line.
// Blocks of parked scenes keep their old values.  The gathers are latency
// bound, so registers are capped at 64 (no spills) for 32 resident warps per
// SM instead of 28; the cap also keeps every tunable CTA size (up to 1024
// threads) within the SM's 65,536 registers.
template <typename HT, typename T>
__global__ void __maxnreg__(64) k_assemble(DeviceBatch b, const HT* __restrict__ elemH, T* __restrict__ lhs) {
  const size_t g = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= (size_t)kSlice * b.nslotRows) return;
  const int r = (int)(g / kSlice), lane = (int)(g % kSlice);
  int u, blk;
  if (slot_block(b, r, lane, u, blk)) {
    const SceneParams& sp = b.scenes[b.vertexScene[u]];
    if (sp.active && !b.solve[b.vertexScene[u]].newtonDone) {
      HT sum[9];
#pragma unroll
      for (int e = 0; e < 9; e++) sum[e] = HT(0);
      // contributions in flight: 4 in FP32, 2 in FP64 (register budget)
      constexpr int kQ = sizeof(HT) == sizeof(float) ? 4 : 2;
      const int k0 = b.blkptr[blk], k1 = b.blkptr[blk + 1];
      for (int k = k0; k < k1; k += kQ) {
        int src[kQ];
#pragma unroll
        for (int q = 0; q < kQ; q++) src[q] = (k + q < k1) ? __ldg(&b.blksrc[k + q]) : 0;
        HT val[kQ][9];
#pragma unroll
        for (int q = 0; q < kQ; q++) {
          const int t = src[q] >> 4, ea = (src[q] >> 2) & 3, eb = src[q] & 3;
          const int off = 9 * ((ea <= eb) ? upper_block(ea, eb) : upper_block(eb, ea));
          if (sizeof(HT) == sizeof(float)) {
            // the block's 9 values from the three 16-byte words that cover
            // them (the tet's record starts on a 16-byte boundary), then
            // shifted down by the block's offset within the first word
            const float4* W = reinterpret_cast<const float4*>(elemH + (size_t)kElemHessStride * t + (off & ~3));
            float4 w0 = make_float4(0.f, 0.f, 0.f, 0.f), w1 = w0, w2 = w0;
            if (k + q < k1) {
              w0 = __ldg(W);
              w1 = __ldg(W + 1);
              w2 = __ldg(W + 2);
            }
            const float win[12] = {w0.x, w0.y, w0.z, w0.w, w1.x, w1.y, w1.z, w1.w, w2.x, w2.y, w2.z, w2.w};
            const int sh = off & 3;
            float mid[11];
#pragma unroll
            for (int e = 0; e < 11; e++) mid[e] = (sh & 1) ? win[e + 1] : win[e];
#pragma unroll
            for (int e = 0; e < 9; e++) val[q][e] = HT((sh & 2) ? mid[e + 2] : mid[e]);
          } else {
            const HT* H = elemH + (size_t)kElemHessStride * t + off;
#pragma unroll
            for (int e = 0; e < 9; e++) val[q][e] = (k + q < k1) ? H[e] : HT(0);
          }
          if (ea > eb) {  // lower-triangle block: the stored upper block transposed
            HT tmp;
            tmp = val[q][1]; val[q][1] = val[q][3]; val[q][3] = tmp;
            tmp = val[q][2]; val[q][2] = val[q][6]; val[q][6] = tmp;
            tmp = val[q][5]; val[q][5] = val[q][7]; val[q][7] = tmp;
          }
        }
#pragma unroll
        for (int q = 0; q < kQ; q++)
          if (k + q < k1)
#pragma unroll
            for (int e = 0; e < 9; e++) sum[e] += val[q][e];
      }
      const int w = b.cols[blk];
      const double dt = sp.dt;
      const bool fu = b.freeMask[u] != 0, fw = b.freeMask[w] != 0;
      T* out = lhs + (size_t)r * kSlotVals + lane;
      if (sp.integrator == kIntegratorPosition) {
        // A = M (1/dt^2 - alpha/dt) - (beta/dt) K0 - K (BACKWARD_EULER_POSITION.cpp:207)
        const double invDt = 1.0 / dt;
        const HT m = fu ? HT(b.mass[u] * (invDt * invDt - sp.rayAlpha * invDt)) : HT(1);
        const HT cK0 = HT(-(sp.rayBeta * invDt));
        const double* K0 = b.K0 + 9 * (size_t)blk;
#pragma unroll
        for (int e = 0; e < 9; e++) {
          HT val = (fu && fw) ? cK0 * HT(K0[(e / 3) + 3 * (e % 3)]) - sum[e] : HT(0);
          if (u == w && e % 4 == 0) val += m;
          out[kSlice * e] = T(val);
        }
      } else if (sp.integrator == kIntegratorNewmark) {
        // A = alpha_0 M - K (NEWMARK.cpp:262; its C is zeroed before use)
        const HT m = fu ? HT(sp.nm[0] * b.mass[u]) : HT(1);
#pragma unroll
        for (int e = 0; e < 9; e++) {
          HT val = (fu && fw) ? -sum[e] : HT(0);
          if (u == w && e % 4 == 0) val += m;
          out[kSlice * e] = T(val);
        }
      } else {
        const HT m = fu ? HT(b.mass[u]) : HT(1);
        const HT ndt2 = HT(-(dt * dt));
#pragma unroll
        for (int e = 0; e < 9; e++) {
          HT val = (fu && fw) ? ndt2 * sum[e] : HT(0);
          if (u == w && e % 4 == 0) val += m;
          out[kSlice * e] = T(val);
        }
      }
    }
  }
}

// Raw K blocks (column major) and R: the reference's stiffness and force
// outputs (TET_MESH_FASTER.cpp:89-133, TET_MESH.cpp:736-770) for inspection.
__global__ void k_assemble_raw(DeviceBatch b, double* K, double* R) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < 9L * b.nblocks) {
    const int blk = (int)(g / 9), e = (int)(g % 9);
    const int r = e / 3, c = e % 3;
    K[9 * (size_t)blk + r + 3 * c] = gather_block_entry(b, b.elemH, blk, r, c);
  }
  if (g < 3L * b.nv) {
    const int u = (int)(g / 3), i = (int)(g % 3);
    double acc = 0.0;
    for (int k = b.vtxptr[u]; k < b.vtxptr[u + 1]; k++) {
      const int inc = b.vtxinc[k];
      acc += b.elemG[12 * (size_t)(inc >> 2) + 3 * (inc & 3) + i];
    }
    R[g] = acc;
  }
}

// Preconditioner from LHS's diagonal blocks: 3x3 inverse (block Jacobi) or
// 1/diag (Jacobi, BasicPreconditioners.h:67-75; zero diagonal -> 1).
template <typename T>
__global__ void k_diag_inverse(DeviceBatch b, const T* __restrict__ lhs, T* __restrict__ minv, int precond) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv || !b.scenes[b.vertexScene[u]].active || b.solve[b.vertexScene[u]].newtonDone) return;
  int k = b.rowptr[u];
  while (b.cols[k] != u) k++;
  const T* Lu = lhs + lhs_slot(b, u, k - b.rowptr[u]);
  double D[9];
#pragma unroll
  for (int i = 0; i < 9; i++) D[i] = (double)Lu[kSlice * i];
  if (b.collOn) {  // the vertex's own contact block (FP64, beside the LHS)
#pragma unroll
    for (int i = 0; i < 9; i++) D[i] += b.coll.diag[9 * (size_t)u + i];
  }
  T* M = minv + 9 * (size_t)u;
  if (precond == 1) {
    const double c00 = D[4] * D[8] - D[5] * D[7];
    const double c01 = D[5] * D[6] - D[3] * D[8];
    const double c02 = D[3] * D[7] - D[4] * D[6];
    const double det = D[0] * c00 + D[1] * c01 + D[2] * c02;
    const double id = 1.0 / det;
    M[0] = T(c00 * id);
    M[1] = T((D[2] * D[7] - D[1] * D[8]) * id);
    M[2] = T((D[1] * D[5] - D[2] * D[4]) * id);
    M[3] = T(c01 * id);
    M[4] = T((D[0] * D[8] - D[2] * D[6]) * id);
    M[5] = T((D[2] * D[3] - D[0] * D[5]) * id);
    M[6] = T(c02 * id);
    M[7] = T((D[1] * D[6] - D[0] * D[7]) * id);
    M[8] = T((D[0] * D[4] - D[1] * D[3]) * id);
  } else {
#pragma unroll
    for (int i = 0; i < 9; i++) M[i] = T(0);
#pragma unroll
    for (int i = 0; i < 3; i++) M[4 * i] = T(D[4 * i] != 0.0 ? 1.0 / D[4 * i] : 1.0);
  }
}

// rhs = S dt (sum_e g_e + f_ext) per vertex (element g already carries
// dt (f + dt He v)); y = 0; r64 = rhs.  Per scene: |rhs|^2 and the FP64
// stopping threshold; an all-zero right-hand side finishes the solve (x = 0).
template <int TV>
__global__ void __launch_bounds__(TV) k_rhs(DeviceBatch b) {
  __shared__ double sh[TV / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  if (!b.scenes[s].active) {  // parked scene: nothing to solve this step
    if (tile == b.scenes[s].tile0 && threadIdx.x == 0) {
      SolveState& st = b.solve[s];
      st.outerDone = 1;
      st.converged = 1;
      st.totalIters = 0;
      st.sweep = 0;
    }
    return;
  }
  if (b.solve[s].newtonDone) {  // Newmark: this scene's Newton loop is over
    const int u = b.tileV0[tile] + threadIdx.x;
    if (u < b.tileV1[tile])
#pragma unroll
      for (int i = 0; i < 3; i++) b.y[3 * u + i] = 0.0;
    if (tile == b.scenes[s].tile0 && threadIdx.x == 0) b.solve[s].outerDone = 1;
    return;
  }
  const int u = b.tileV0[tile] + threadIdx.x;
  double rr = 0;
  if (u < b.tileV1[tile]) {
    const double dt = b.scenes[s].dt;
    double acc[3] = {0.0, 0.0, 0.0};
    const int k1 = b.vtxptr[u + 1];
    for (int k = b.vtxptr[u]; k < k1; k += 8) {  // eight incidences in flight, summed in order
      int inc[8];
#pragma unroll
      for (int q = 0; q < 8; q++) inc[q] = (k + q < k1) ? __ldg(&b.vtxinc[k + q]) : 0;
      double gv[8][3];
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const double* g = b.elemG + 12 * (size_t)(inc[q] >> 2) + 3 * (inc[q] & 3);
#pragma unroll
        for (int i = 0; i < 3; i++) gv[q][i] = (k + q < k1) ? g[i] : 0.0;
      }
#pragma unroll
      for (int q = 0; q < 8; q++)
        if (k + q < k1)
#pragma unroll
          for (int i = 0; i < 3; i++) acc[i] += gv[q][i];
    }
    const bool fu = b.freeMask[u] != 0;
    if (b.collOn && fu) {  // collision tets: dt (f + dt H v), in pair order
      for (int k = b.coll.incCount[u]; k < b.coll.incCount[u + 1]; k++) {
        const int e = b.coll.incList[k];
        const double* g = b.coll.pairRhs + 12 * (size_t)(e >> 2) + 3 * (e & 3);
#pragma unroll
        for (int i = 0; i < 3; i++) acc[i] += g[i];
      }
    }
    double bi[3];
    if (b.scenes[s].integrator == kIntegratorPosition) {
      // b = (M/dt - C) v + R + f_ext with C = alpha M + beta K0
      // (BACKWARD_EULER_POSITION.cpp:196; K0 at zero displacement,
      // TIMESTEPPER.cpp:213-236)
      const SceneParams& sp = b.scenes[s];
      const double invDt = 1.0 / dt, m = b.mass[u];
      double k0v[3] = {0.0, 0.0, 0.0};
      for (int k = b.rowptr[u]; k < b.rowptr[u + 1]; k++) {
        const double* blk = b.K0 + 9 * (size_t)k;
        const int w = b.cols[k];
#pragma unroll
        for (int i = 0; i < 3; i++)
#pragma unroll
          for (int c = 0; c < 3; c++) k0v[i] += blk[i + 3 * c] * b.v[3 * w + c];
      }
#pragma unroll
      for (int i = 0; i < 3; i++)
        bi[i] = (invDt - sp.rayAlpha) * m * b.v[3 * u + i] - sp.rayBeta * k0v[i] + acc[i] + b.fext[3 * u + i];
    } else if (b.scenes[s].integrator == kIntegratorNewmark) {
      // b = M (a0 (x - x_old) - a2 a_old - a1 v_old) - R - f_ext (NEWMARK.cpp:244-255; C = 0)
      const double* nm = b.scenes[s].nm;
      const double m = b.mass[u];
#pragma unroll
      for (int i = 0; i < 3; i++) {
        const size_t q = 3 * (size_t)u + i;
        const double t = m * (nm[0] * (b.x[q] - b.xOld[q]) - nm[2] * b.aOld[q] - nm[1] * b.vOld[q]);
        bi[i] = t - acc[i] - b.fext[q];
      }
    } else {
      // b = dt (R + dt K v + f_ext); acc holds dt (R + dt K v)
#pragma unroll
      for (int i = 0; i < 3; i++) bi[i] = acc[i] + dt * b.fext[3 * u + i];
    }
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double ri = fu ? bi[i] : 0.0;
      b.rhs[3 * u + i] = ri;
      b.r64[3 * u + i] = ri;
      b.y[3 * u + i] = 0.0;
      rr += ri * ri;
    }
  }
  const double t = block_sum<TV>(rr, sh);
  if (threadIdx.x == 0) b.partial[kPartials * tile] = t;
  SolveState& st = b.solve[s];
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketB, sp.ntiles, &flag)) return;
  const double srr = sum_partials<TV>(b.partial, sp.tile0, sp.ntiles, 0, sh);
  if (threadIdx.x == 0) {
    st.rhsNorm2 = srr;
    st.newtonR = srr;  // Newmark's maxR = |rhs|^2 (NEWMARK.cpp:275)
    st.threshold = fmax(st.tol * st.tol * srr, DBL_MIN);
    st.rr64 = srr;
    st.rScale = pow2_near_norm(srr);
    st.sweep = 0;
    st.totalIters = 0;
    st.converged = 0;
    st.outerDone = 0;
    if (srr == 0.0) {  // ConjugateGradient.h:49-55
      st.outerDone = 1;
      st.converged = 1;
    } else if (!finite(srr)) {
      st.outerDone = 1;
      st.converged = -1;
    }
  }
}

__global__ void k_set_active(DeviceBatch b) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *b.active = b.nTileScenes;  // cluster scenes never count
}

// Start of one inner solve on r_T = (T) r64: d = 0, p = s = 0, u = Minv r,
// gamma = (r, u), |r|^2.  Inner tolerance: the outer one for FP64; for FP32
// the relative reduction still needed, floored at the inner tolerance
// (default 1e-5: FP32 stagnation).
template <int TV, typename T>
__global__ void __launch_bounds__(TV) k_inner_init(DeviceBatch b, PcgVecs<T> v) {
  __shared__ double sh[TV / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  SolveState& st = b.solve[s];
  const SceneParams& sp = b.scenes[s];
  if (sp.pcgCluster) return;  // solved by its cluster, concurrently (cluster_pcg.cu)
  if (st.outerDone) {
    // this scene's solve is over: mark the inner solve done once
    if (tile == sp.tile0 && threadIdx.x == 0) {
      st.done = 1;
      atomicSub(b.active, 1);
    }
    return;
  }
  const int u = b.tileV0[tile] + threadIdx.x;
  const double sc = (sizeof(T) != sizeof(double) && st.rScale > 0.0) ? st.rScale : 1.0;
  const double inv = 1.0 / sc;  // exact: sc is a power of two
  T rr = T(0), ru = T(0);
  if (u < b.tileV1[tile]) {
    T r3[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      r3[i] = T(b.r64[3 * u + i] * inv);
      if (sizeof(T) != sizeof(double)) v.r[3 * u + i] = r3[i];
      v.d[3 * u + i] = T(0);
      v.p[3 * u + i] = T(0);
      v.s[3 * u + i] = T(0);
      rr += r3[i] * r3[i];
    }
    const T* M = v.minv + 9 * (size_t)u;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const T ui = M[3 * i] * r3[0] + M[3 * i + 1] * r3[1] + M[3 * i + 2] * r3[2];
      v.u[3 * u + i] = ui;
      ru += r3[i] * ui;
    }
  }
  const double trr = block_sum<TV>(rr, sh);
  const double tru = block_sum<TV>(ru, sh);
  if (threadIdx.x == 0) {
    b.partial[kPartials * tile] = trr;
    b.partial[kPartials * tile + 1] = tru;
  }
  if (!last_tile(&st.ticketB, sp.ntiles, &flag)) return;
  const double srr = sum_partials<TV>(b.partial, sp.tile0, sp.ntiles, 0, sh);
  const double sru = sum_partials<TV>(b.partial, sp.tile0, sp.ntiles, 1, sh);
  if (threadIdx.x == 0) {
    double itol = st.tol;
    if (sizeof(T) != sizeof(double)) itol = fmax(st.tol * sqrt(st.rhsNorm2 / fmax(srr * sc * sc, DBL_MIN)), st.innerFloor);
    st.rr = srr;
    st.gamma = sru;
    st.gammaOld = 1.0;
    st.alpha = 1.0;
    st.beta = 0.0;
    st.alphaF = 1.0f;
    st.betaF = 0.0f;
    st.iters = 0;
    st.innerThreshold = fmax(itol * itol * srr, DBL_MIN);
    st.done = 0;
    if (srr == 0.0 || srr < st.innerThreshold) {
      st.done = 1;
      atomicSub(b.active, 1);
    }
  }
}

// Row i of vertex u of w H_coll x (w = collision_lhs_scale), H_coll = sum over the
// vertex's collision tets of (c c^T) (x) G (free rows only; x vanishes on
// pinned rows, which keeps the columns masked too).  FP64 throughout: the
// contact blocks are not part of the (possibly FP32) assembled LHS.
template <typename T>
__device__ __forceinline__ double collision_row(const DeviceBatch& b, int u, int i, const T* __restrict__ x) {
  const DeviceCollisions& c = b.coll;
  const int k0 = c.incCount[u], k1 = c.incCount[u + 1];
  if (k0 == k1) return 0.0;
  const double scale = collision_lhs_scale(b, b.vertexScene[u]);
  double acc = 0.0;
  for (int k = k0; k < k1; k++) {
    const int e = c.incList[k], p = e >> 2, a = e & 3;
    const int4 ct = c.pairTet[p];
    const double* C = c.pairC + 4 * (size_t)p;
    const double* G = c.pairG + 9 * (size_t)p;
    const int id[4] = {ct.x, ct.y, ct.z, ct.w};
    double z[3] = {0.0, 0.0, 0.0};
#pragma unroll
    for (int q = 0; q < 4; q++)
#pragma unroll
      for (int j = 0; j < 3; j++) z[j] += C[q] * double(x[3 * id[q] + j]);
    acc += C[a] * (G[i] * z[0] + G[i + 3] * z[1] + G[i + 6] * z[2]);
  }
  return scale * acc;
}

// Threads of an SpMV CTA: one per vertex in FP32 (the sliced LHS makes
// every matrix and column load of a warp one line, and a vertex's three rows
// share its column loads and u gathers); one per scalar row in FP64, whose
// SpMV is bound by GB300's narrow FP64 pipe and wants three times the warps
// to keep it fed.
template <typename T>
__host__ __device__ constexpr int spmv_threads(int TV) { return sizeof(T) == sizeof(float) ? TV : 3 * TV; }

// The scene's iteration step in its last SpMV CTA (thread 0), from
// rho = |r|^2, gamma = (r, u) and delta = (w, u): after an update, stop when
// |r|^2 < threshold (ConjugateGradient.h:75-78), on a non-finite value, or at
// the iteration limit; otherwise beta and alpha for this iteration's update,
// which the iteration count then includes.
template <typename T>
__device__ __forceinline__ void spmv_decide(const DeviceBatch& b, SolveState& st, double rho, double gamma,
                                            double delta) {
  // a negative threshold marks the kernel timing of hobak_batch_time_kernels,
  // which repeats the SpMV on fixed vectors: the scalars stay as they are
  if (st.innerThreshold < 0.0) return;
  if (st.iters > 0) {
    st.rr = rho;
    bool stop = false;
    if (rho < st.innerThreshold) {
      stop = true;
    } else if (!finite(rho) || !finite(gamma) || !finite(st.alpha)) {
      stop = true;
      st.converged = -1;
      st.outerDone = 1;
    } else if (st.totalIters >= st.maxit) {
      stop = true;
    }
    if (stop) {
      st.done = 1;
      atomicSub(b.active, 1);
      if (sizeof(T) == sizeof(double) && st.converged >= 0) {
        // FP64 path: the recursive residual is the solver's verdict (Eigen)
        st.rr64 = rho;
        st.converged = rho < st.threshold ? 1 : 0;
        st.outerDone = 1;
      }
      return;
    }
  }
  st.delta = delta;
  if (st.iters == 0) {
    st.beta = 0.0;
    st.alpha = gamma / delta;
  } else {
    const double beta = gamma / st.gamma;  // st.gamma: the previous iteration's (r, u)
    st.beta = beta;
    st.alpha = gamma / (delta - beta * gamma / st.alpha);
  }
  st.gammaOld = st.gamma;
  st.gamma = gamma;
  st.alphaF = float(st.alpha);
  st.betaF = float(st.beta);
  st.iters += 1;
  st.totalIters += 1;
}

// FP64: w = A u, one thread per scalar row (9 DFMA per block over the row's
// three threads), and delta = (w, u).  In the sliced LHS the row's entries
// of block j sit at kSlice * (3 i + c) past the slot, so a warp's 30 rows
// (10 vertices) read three lines per load.
template <int TV, typename T>
__device__ __forceinline__ void spmv_tile_rows(const DeviceBatch& b, const PcgVecs<T>& v, int tile, double* sh,
                                               int* flag) {
  // before the dependency wait: what the previous kernel does not write
  const int s = b.tileScene[tile];
  const int row = 3 * b.tileV0[tile] + threadIdx.x;
  const bool valid = row < 3 * b.tileV1[tile];
  const int u = row / 3, i = row - 3 * u;
  int len = 0;
  size_t mb = 0, cb = 0;
  int wn[4] = {0, 0, 0, 0};
  if (valid) {
    len = b.rowptr[u + 1] - b.rowptr[u];
    mb = lhs_slot(b, u, 0) + kSlice * 3 * i;
    cb = col_slot(b, u, 0);
#pragma unroll
    for (int q = 0; q < 4; q++) wn[q] = (q < len) ? __ldg(&b.colS[cb + kSlice * q]) : 0;
  }
  pdl_wait();
  SolveState& st = b.solve[s];
  if (st.done) return;
  const T* __restrict__ r = (sizeof(T) == sizeof(double)) ? reinterpret_cast<const T*>(b.r64) : v.r;
  T dl = T(0), gl = T(0), rl = T(0);
  if (valid) {
    const T* __restrict__ uu = v.u;
    // Four blocks per trip, all their loads issued together (predicated past
    // the row's end); the next trip's columns are fetched one trip ahead.
    // Two FMA chains: 3 FMA per block, the FP64 minimum.
    T acc0 = T(0), acc1 = T(0);
    for (int j = 0; j < len; j += 4) {
      int w[4];
#pragma unroll
      for (int q = 0; q < 4; q++) {
        w[q] = wn[q];
        wn[q] = (j + 4 + q < len) ? __ldg(&b.colS[cb + kSlice * (j + 4 + q)]) : 0;
      }
#pragma unroll
      for (int q = 0; q < 4; q++) {
        if (j + q < len) {
          const T* B = v.lhs + mb + (size_t)kSlotVals * (j + q);
          T& acc = (q & 1) ? acc1 : acc0;
          acc = fma(__ldg(&B[0]), __ldg(&uu[3 * w[q]]), acc);
          acc = fma(__ldg(&B[kSlice]), __ldg(&uu[3 * w[q] + 1]), acc);
          acc = fma(__ldg(&B[2 * kSlice]), __ldg(&uu[3 * w[q] + 2]), acc);
        }
      }
    }
    T acc = acc0 + acc1;
    if (b.collOn && b.freeMask[u]) acc += T(collision_row<T>(b, u, i, uu));
    v.w[row] = acc;
    const T ui = uu[row], ri = r[row];
    dl = acc * ui;
    gl = ri * ui;
    rl = ri * ri;
  }
  double t[3];
  block_sum3<3 * TV>(rl, gl, dl, sh, t);
  if (threadIdx.x == 0) {
    b.partial[kPartials * tile] = t[0];
    b.partial[kPartials * tile + 1] = t[1];
    b.partial[kPartials * tile + 2] = t[2];
  }
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketA, sp.ntiles, flag)) return;
  double tot[3];
  sum_partials3<3 * TV>(b.partial, sp.tile0, sp.ntiles, sh, tot);
  if (threadIdx.x == 0) spmv_decide<T>(b, st, tot[0], tot[1], tot[2]);
}

// FP32: w = A u, one thread per vertex (its three rows; 9 FMA per block), and
// delta = (w, u); the scene's last CTA forms beta and alpha.  The warps run
// over 32 consecutive vertices, so in the sliced LHS every matrix and column
// load of a warp is one contiguous line.
template <int TV, typename T>
__device__ __forceinline__ void spmv_tile(const DeviceBatch& b, const PcgVecs<T>& v, int tile, double* sh, int* flag) {
  // before the dependency wait: what the previous kernel does not write
  const int s = b.tileScene[tile];
  const int u = b.tileV0[tile] + threadIdx.x;
  const bool valid = u < b.tileV1[tile];
  int len = 0;
  size_t mb = 0, cb = 0;
  constexpr int Q0 = sizeof(T) == sizeof(float) ? 4 : 2;
  int wn[Q0];
#pragma unroll
  for (int q = 0; q < Q0; q++) wn[q] = 0;
  if (valid) {
    len = b.rowptr[u + 1] - b.rowptr[u];
    mb = lhs_slot(b, u, 0);
    cb = col_slot(b, u, 0);
#pragma unroll
    for (int q = 0; q < Q0; q++) wn[q] = (q < len) ? __ldg(&b.colS[cb + kSlice * q]) : 0;
  }
  pdl_wait();
  SolveState& st = b.solve[s];
  // the done test waits for its load only after the first trip's loads are
  // in flight
  const int done = st.done;
  T dl = T(0), gl = T(0), rl = T(0);
  if (valid) {
    const T* __restrict__ uu = v.u;
    // Q blocks per trip (4 in FP32, 2 in FP64: register budget), all their
    // loads issued together (predicated past the row's end); the next trip's
    // columns are fetched one trip ahead, so each trip waits on one memory
    // latency (the u gather) instead of two.
    constexpr int Q = sizeof(T) == sizeof(float) ? 4 : 2;
    T a0 = T(0), a1 = T(0), a2 = T(0);
    for (int j = 0; j < len; j += Q) {
      int w[Q];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        w[q] = wn[q];
        wn[q] = (j + Q + q < len) ? __ldg(&b.colS[cb + kSlice * (j + Q + q)]) : 0;
      }
      T x[Q][3], m[Q][9];
#pragma unroll
      for (int q = 0; q < Q; q++) {
        const T* B = v.lhs + mb + (size_t)kSlotVals * (j + q);
#pragma unroll
        for (int e = 0; e < 9; e++) m[q][e] = (j + q < len) ? __ldg(&B[kSlice * e]) : T(0);
#pragma unroll
        for (int c = 0; c < 3; c++) x[q][c] = (j + q < len) ? __ldg(&uu[3 * w[q] + c]) : T(0);
      }
      if (done) return;
#pragma unroll
      for (int q = 0; q < Q; q++) {
        if (j + q < len) {
          a0 = fma(m[q][0], x[q][0], fma(m[q][1], x[q][1], fma(m[q][2], x[q][2], a0)));
          a1 = fma(m[q][3], x[q][0], fma(m[q][4], x[q][1], fma(m[q][5], x[q][2], a1)));
          a2 = fma(m[q][6], x[q][0], fma(m[q][7], x[q][1], fma(m[q][8], x[q][2], a2)));
        }
      }
    }
    if (b.collOn && b.freeMask[u]) {
      a0 += T(collision_row<T>(b, u, 0, uu));
      a1 += T(collision_row<T>(b, u, 1, uu));
      a2 += T(collision_row<T>(b, u, 2, uu));
    }
    v.w[3 * u] = a0;
    v.w[3 * u + 1] = a1;
    v.w[3 * u + 2] = a2;
    const T u0 = uu[3 * u], u1 = uu[3 * u + 1], u2 = uu[3 * u + 2];
    const T r0 = v.r[3 * u], r1 = v.r[3 * u + 1], r2 = v.r[3 * u + 2];
    dl = a0 * u0 + a1 * u1 + a2 * u2;
    gl = r0 * u0 + r1 * u1 + r2 * u2;
    rl = r0 * r0 + r1 * r1 + r2 * r2;
  }
  if (done) return;  // threads without rows (the CTA returns as one)
  double t[3];
  block_sum3<TV>(rl, gl, dl, sh, t);
  if (threadIdx.x == 0) {
    b.partial[kPartials * tile] = t[0];
    b.partial[kPartials * tile + 1] = t[1];
    b.partial[kPartials * tile + 2] = t[2];
  }
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketA, sp.ntiles, flag)) return;
  double tot[3];
  sum_partials3<TV>(b.partial, sp.tile0, sp.ntiles, sh, tot);
  if (threadIdx.x == 0) spmv_decide<T>(b, st, tot[0], tot[1], tot[2]);
}

// CTA -> tile of the PCG loop kernels (grid = all tiles).  While every scene
// iterates, CTA i takes tile i; once scenes have finished, the CTAs take the
// compacted list of tiles still iterating (k_compact_tiles) and the rest exit
// after a single load instead of walking tile -> scene -> solve state.
__device__ __forceinline__ int loop_tile(const DeviceBatch& b) {
  const int n = *b.nLoopTiles;
  if (n == b.ntiles) return blockIdx.x;
  return (int)blockIdx.x < n ? b.loopTiles[blockIdx.x] : -1;
}

template <int TV, typename T>
__global__ void __launch_bounds__(spmv_threads<T>(TV)) k_spmv(DeviceBatch b, PcgVecs<T> v) {
  __shared__ double sh[3 * spmv_threads<T>(TV) / 32];
  __shared__ int flag;
  pdl_trigger();
  const int tile = loop_tile(b);
  if (tile < 0) return;
  if constexpr (sizeof(T) == sizeof(float)) spmv_tile<TV, T>(b, v, tile, sh, &flag);
  else spmv_tile_rows<TV, T>(b, v, tile, sh, &flag);
}

// p = u + beta p; s = w + beta s; d += alpha p; r -= alpha s; u = Minv r
// (the dot products of the new r and u are the next SpMV's).
template <int TV, typename T>
// One thread per scalar row (three times the threads of a per-vertex loop,
// which a 40^3 scene needs to cover the GPU's latency), 30 rows per warp; the
// 3x3 block of Minv reads its vertex's three new residual rows by shuffles.
__device__ __forceinline__ void update_tile(const DeviceBatch& b, const PcgVecs<T>& v, int tile) {
  // before the dependency wait: what the previous kernel does not write
  const int s = b.tileScene[tile];
  const int lane = threadIdx.x % 32;
  const int row = 3 * b.tileV0[tile] + 30 * (threadIdx.x / 32) + lane;
  const bool valid = lane < 30 && row < 3 * b.tileV1[tile];
  T M0 = T(0), M1 = T(0), M2 = T(0);
  if (valid) {
    const T* M = v.minv + 3 * (size_t)row;  // row i of the vertex's block
    M0 = M[0];
    M1 = M[1];
    M2 = M[2];
  }
  pdl_wait();
  // the solve state and the row's six vectors in one round of loads; the
  // done test comes after them instead of in front (a finished scene's tiles
  // leave the compacted list at the next loop body)
  SolveState& st = b.solve[s];
  const int done = st.done;
  // FP32 scalars come pre-converted: a double-to-float conversion per thread
  // would occupy GB300's narrow FP64 pipe
  T alpha, beta;
  if constexpr (sizeof(T) == sizeof(float)) {
    alpha = st.alphaF;
    beta = st.betaF;
  } else {
    alpha = st.alpha;
    beta = st.beta;
  }
  T* __restrict__ r = (sizeof(T) == sizeof(double)) ? reinterpret_cast<T*>(b.r64) : v.r;
  T u0 = T(0), p0 = T(0), w0 = T(0), s0 = T(0), d0 = T(0), r0 = T(0);
  if (valid) {
    u0 = v.u[row];
    p0 = v.p[row];
    w0 = v.w[row];
    s0 = v.s[row];
    d0 = v.d[row];
    r0 = r[row];
  }
  if (done) return;
  T rnew = T(0);
  if (valid) {
    const T p = u0 + beta * p0;
    const T sv = w0 + beta * s0;
    v.p[row] = p;
    v.s[row] = sv;
    v.d[row] = d0 + alpha * p;
    rnew = r0 - alpha * sv;
    r[row] = rnew;
  }
  // the vertex's three new residual rows sit in lanes base..base+2 of this
  // warp (10 vertices per warp): exchange them by shuffles, no barrier
  const int base = lane - lane % 3;
  const T ra = __shfl_sync(0xffffffffu, rnew, base);
  const T rb = __shfl_sync(0xffffffffu, rnew, base + 1);
  const T rc = __shfl_sync(0xffffffffu, rnew, base + 2);
  if (valid) v.u[row] = M0 * ra + M1 * rb + M2 * rc;
}

template <int TV, typename T>
__global__ void __launch_bounds__(32 * update_warps(TV), TV == 64 ? 8 : 4) k_update(DeviceBatch b, PcgVecs<T> v) {
  pdl_trigger();
  const int tile = loop_tile(b);
  if (tile >= 0) update_tile<TV, T>(b, v, tile);
}

// Compacted list of the tiles whose scene's inner PCG still runs, rebuilt at
// the start of every PCG loop body (one CTA; scenes in order, tiles in order).
// In graph mode it also picks the loop body's grid class: the smallest grid
// that covers the tiles left, so that late iterations with few scenes still
// running do not launch a CTA per tile of the batch.
__global__ void __launch_bounds__(1024) k_compact_tiles(DeviceBatch b, unsigned long long switchHandle,
                                                        GridClasses classes) {
  __shared__ int warpTot[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  const int lane = threadIdx.x % 32, wid = threadIdx.x / 32;
  for (int base = 0; base < b.nscenes; base += 1024) {
    const int s = base + threadIdx.x;
    const int cnt = (s < b.nscenes && !b.solve[s].done && !b.scenes[s].pcgCluster) ? b.scenes[s].ntiles : 0;
    int x = cnt;  // inclusive scan in the warp
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warpTot[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int t = warpTot[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, t, o);
        if (lane >= o) t += y;
      }
      warpTot[lane] = t;  // inclusive over warps
    }
    __syncthreads();
    const int off = carry + (wid > 0 ? warpTot[wid - 1] : 0) + x - cnt;
    if (cnt > 0) {
      const int t0 = b.scenes[s].tile0;
      for (int j = 0; j < cnt; j++) b.loopTiles[off + j] = t0 + j;
    }
    __syncthreads();
    if (threadIdx.x == 0) carry += warpTot[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    *b.nLoopTiles = carry;
    if (switchHandle) {
      int k = 0;
      while (k + 1 < classes.n && classes.grid[k + 1] >= carry) k++;
      cudaGraphSetConditional((cudaGraphConditionalHandle)switchHandle, (unsigned)k);
    }
  }
}

// Mixed precision, after an inner solve: y += d (FP64), one vertex per thread.
__global__ void k_accumulate(DeviceBatch b) {
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  if (b.solve[s].outerDone || b.scenes[s].pcgCluster) return;  // a cluster refines its own scene
  const int u = b.tileV0[tile] + threadIdx.x;
  if (u >= b.tileV1[tile]) return;
  const double sc = b.solve[s].rScale > 0.0 ? b.solve[s].rScale : 1.0;
#pragma unroll
  for (int i = 0; i < 3; i++) b.y[3 * u + i] += sc * double(b.v32.d[3 * u + i]);
}

// Mixed precision: r64 = rhs - A y in FP64 (FP32 matrix entries promoted),
// |r64|^2, then the outer test: converged, out of sweeps, or refine again.
template <int TV>
__global__ void __launch_bounds__(3 * TV) k_residual(DeviceBatch b) {
  __shared__ double sh[3 * TV / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  SolveState& st = b.solve[s];
  if (st.outerDone || b.scenes[s].pcgCluster) return;  // a cluster refines its own scene
  const int row = 3 * b.tileV0[tile] + threadIdx.x;
  double rr = 0.0;
  if (row < 3 * b.tileV1[tile]) {
    const int u = row / 3, i = row - 3 * u;
    const float* A = b.v32.lhs + lhs_slot(b, u, 0) + kSlice * 3 * i;
    double acc = 0.0;
    const int k0 = b.rowptr[u], k1 = b.rowptr[u + 1];
    for (int k = k0; k < k1; k++) {
      const int w = b.cols[k];
      const float* B = A + (size_t)kSlotVals * (k - k0);
      acc += double(B[0]) * b.y[3 * w] + double(B[kSlice]) * b.y[3 * w + 1] + double(B[2 * kSlice]) * b.y[3 * w + 2];
    }
    if (b.collOn && b.freeMask[u]) acc += collision_row<double>(b, u, i, b.y);
    const double ri = b.rhs[row] - acc;
    b.r64[row] = ri;
    rr = ri * ri;
  }
  const double t = block_sum<3 * TV>(rr, sh);
  if (threadIdx.x == 0) b.partial[kPartials * tile + 3] = t;
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketA, sp.ntiles, &flag)) return;
  const double srr = sum_partials<3 * TV>(b.partial, sp.tile0, sp.ntiles, 3, sh);
  if (threadIdx.x == 0) {
    st.rr64 = srr;
    st.rScale = pow2_near_norm(srr);
    st.sweep += 1;
    if (srr < st.threshold) {
      st.outerDone = 1;
      st.converged = 1;
    } else if (!finite(srr)) {
      st.outerDone = 1;
      st.converged = -1;
    } else if (st.sweep >= st.maxSweeps || st.totalIters >= st.maxit) {
      st.outerDone = 1;
      st.converged = 0;
    }
  }
}

// Graph loop control: keep iterating while any scene's inner PCG runs.
__global__ void k_continue(const int* active, unsigned long long* bodyRuns, cudaGraphConditionalHandle h) {
  if (threadIdx.x == 0 && blockIdx.x == 0) {
    *bodyRuns += 1ull;
    cudaGraphSetConditional(h, *active > 0 ? 1u : 0u);
  }
}

// Velocity integrator: v += y; x += dt v; v = S v
// (BACKWARD_EULER_VELOCITY.cpp:191-201).  Position integrator: x += y;
// v = (x - x_old) / dt; v = S v (BACKWARD_EULER_POSITION.cpp:241-301).
__global__ void k_finish_step(DeviceBatch b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv || !b.scenes[b.vertexScene[u]].active) return;
  const SceneParams& sp = b.scenes[b.vertexScene[u]];
  const double dt = sp.dt;
  const bool fu = b.freeMask[u] != 0;
  if (sp.integrator == kIntegratorPosition) {
    const double invDt = 1.0 / dt;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double xo = b.x[3 * u + i], xn = xo + b.y[3 * u + i];
      b.x[3 * u + i] = xn;
      b.v[3 * u + i] = fu ? invDt * (xn - xo) : 0.0;
    }
    return;
  }
  if (sp.integrator == kIntegratorNewmark) {
    // v = a3 dx + a4 v_old + a5 a_old, a = a0 dx - a1 v_old - a2 a_old, S
    // (NEWMARK.cpp:321-333); x itself was updated by the Newton loop
    const double* nm = sp.nm;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const size_t q = 3 * (size_t)u + i;
      const double dx = b.x[q] - b.xOld[q];
      const double vn = nm[3] * dx + nm[4] * b.vOld[q] + nm[5] * b.aOld[q];
      const double an = nm[0] * dx - nm[1] * b.vOld[q] - nm[2] * b.aOld[q];
      b.v[q] = fu ? vn : 0.0;
      b.acc[q] = fu ? an : 0.0;
    }
    return;
  }
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const double vn = b.v[3 * u + i] + b.y[3 * u + i];
    b.x[3 * u + i] = b.x[3 * u + i] + dt * vn;
    b.v[3 * u + i] = fu ? vn : 0.0;
  }
}

}  // namespace

void launch_begin_step(const DeviceBatch& b, cudaStream_t s) {
  k_begin_step<<<(b.nv + 255) / 256, 256, 0, s>>>(b);
}

template <typename T>
void launch_assemble(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s) {
  if (b.nblocks == 0) return;
  if (sizeof(T) == sizeof(double)) {
    const size_t n = (size_t)kSlotVals * b.nslotRows;
    k_assemble_entry<double, T><<<(unsigned)((n + b.asmThreads - 1) / b.asmThreads), b.asmThreads, 0, s>>>(
        b, b.elemH, v.lhs);
  } else {
    const size_t n = (size_t)kSlice * b.nslotRows;
    k_assemble<float, T><<<(unsigned)((n + b.asmThreads - 1) / b.asmThreads), b.asmThreads, 0, s>>>(
        b, b.elemHf, v.lhs);
  }
}

void launch_assemble_raw(const DeviceBatch& b, double* K, double* R, cudaStream_t s) {
  const long n = std::max(9L * b.nblocks, 3L * b.nv);
  k_assemble_raw<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, K, R);
}

template <typename T>
void launch_diag_inverse(const DeviceBatch& b, const PcgVecs<T>& v, int precond, cudaStream_t s) {
  k_diag_inverse<T><<<(b.nv + 255) / 256, 256, 0, s>>>(b, v.lhs, v.minv, precond);
}

// PCG loop kernel launch; with `pdl` the kernel may start while the previous
// kernel in the stream drains (programmatic stream serialisation; the kernel
// itself waits with pdl_wait before reading what that kernel writes).
template <typename... KArgs, typename... Args>
void launch_loop_kernel(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s, bool pdl, Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = attr;
  cfg.numAttrs = pdl ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, args...);
}

// Tile-kernel launches dispatch on the batch's tile size.
#define HOBAK_TILE_LAUNCH(KERNEL, THREADS_PER_V, ...)                                   \
  do {                                                                                  \
    if (b.tileV == 64) KERNEL<64><<<b.ntiles, (THREADS_PER_V) * 64, 0, s>>>(__VA_ARGS__);     \
    else KERNEL<128><<<b.ntiles, (THREADS_PER_V) * 128, 0, s>>>(__VA_ARGS__);                 \
  } while (0)

void launch_rhs(const DeviceBatch& b, cudaStream_t s) { HOBAK_TILE_LAUNCH(k_rhs, 1, b); }

void launch_set_active(const DeviceBatch& b, cudaStream_t s) { k_set_active<<<1, 32, 0, s>>>(b); }

GridClasses grid_classes(int ntiles) {
  GridClasses c{};
  c.n = 1;
  c.grid[0] = ntiles;
  for (int g : {4096, 1024, 256, 64})
    if (g < c.grid[c.n - 1] && c.n < kGridClasses) c.grid[c.n++] = g;
  return c;
}

void launch_compact_tiles(const DeviceBatch& b, cudaStream_t s, unsigned long long switchHandle,
                          const GridClasses* classes) {
  const GridClasses c = classes ? *classes : grid_classes(b.ntiles);
  k_compact_tiles<<<1, 1024, 0, s>>>(b, switchHandle, c);
}

template <typename T>
void launch_inner_init(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s) {
  if (b.tileV == 64) k_inner_init<64, T><<<b.ntiles, 64, 0, s>>>(b, v);
  else k_inner_init<128, T><<<b.ntiles, 128, 0, s>>>(b, v);
}

template <typename T>
void launch_spmv(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s, bool pdl, int grid) {
  if (grid <= 0) grid = b.ntiles;
  if (b.tileV == 64) launch_loop_kernel(k_spmv<64, T>, grid, spmv_threads<T>(64), s, pdl, b, v);
  else launch_loop_kernel(k_spmv<128, T>, grid, spmv_threads<T>(128), s, pdl, b, v);
}

template <typename T>
void launch_update(const DeviceBatch& b, const PcgVecs<T>& v, cudaStream_t s, bool pdl, int grid) {
  if (grid <= 0) grid = b.ntiles;
  if (b.tileV == 64) launch_loop_kernel(k_update<64, T>, grid, 32 * update_warps(64), s, pdl, b, v);
  else launch_loop_kernel(k_update<128, T>, grid, 32 * update_warps(128), s, pdl, b, v);
}

void launch_refine(const DeviceBatch& b, cudaStream_t s) {
  k_accumulate<<<b.ntiles, b.tileV, 0, s>>>(b);
  HOBAK_TILE_LAUNCH(k_residual, 3, b);
}

void launch_continue(const DeviceBatch& b, unsigned long long handle, cudaStream_t s) {
  k_continue<<<1, 32, 0, s>>>(b.active, b.bodyRuns, (cudaGraphConditionalHandle)handle);
}
void launch_newton_begin(const DeviceBatch& b, cudaStream_t s) { k_newton_begin<<<1, 256, 0, s>>>(b); }

void launch_newton_update(const DeviceBatch& b, cudaStream_t s) {
  k_newton_step<<<(b.nv + 255) / 256, 256, 0, s>>>(b);
  k_newton_test<<<1, 256, 0, s>>>(b);
}

__global__ void k_set_condition(cudaGraphConditionalHandle h, unsigned value) {
  if (threadIdx.x == 0 && blockIdx.x == 0) cudaGraphSetConditional(h, value);
}

void launch_set_condition(unsigned long long handle, unsigned value, cudaStream_t s) {
  k_set_condition<<<1, 32, 0, s>>>((cudaGraphConditionalHandle)handle, value);
}

void launch_newton_continue(const DeviceBatch& b, unsigned long long handle, cudaStream_t s) {
  k_newton_continue<<<1, 32, 0, s>>>(b.newtonActive, b.newtonRuns, (cudaGraphConditionalHandle)handle);
}

void launch_finish_step(const DeviceBatch& b, cudaStream_t s) {
  k_finish_step<<<(b.nv + 255) / 256, 256, 0, s>>>(b);
}

template void launch_assemble<double>(const DeviceBatch&, const PcgVecs<double>&, cudaStream_t);
template void launch_assemble<float>(const DeviceBatch&, const PcgVecs<float>&, cudaStream_t);
template void launch_diag_inverse<double>(const DeviceBatch&, const PcgVecs<double>&, int, cudaStream_t);
template void launch_diag_inverse<float>(const DeviceBatch&, const PcgVecs<float>&, int, cudaStream_t);
template void launch_inner_init<double>(const DeviceBatch&, const PcgVecs<double>&, cudaStream_t);
template void launch_inner_init<float>(const DeviceBatch&, const PcgVecs<float>&, cudaStream_t);
template void launch_spmv<double>(const DeviceBatch&, const PcgVecs<double>&, cudaStream_t, bool, int);
template void launch_spmv<float>(const DeviceBatch&, const PcgVecs<float>&, cudaStream_t, bool, int);
template void launch_update<double>(const DeviceBatch&, const PcgVecs<double>&, cudaStream_t, bool, int);
template void launch_update<float>(const DeviceBatch&, const PcgVecs<float>&, cudaStream_t, bool, int);

}  // namespace hobak
