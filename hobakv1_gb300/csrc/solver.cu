// Assembly, right-hand side and block-Jacobi PCG kernels (FP64 path).
//
// System of one BACKWARD_EULER_VELOCITY step (BACKWARD_EULER_VELOCITY.cpp:157-176):
//   b   = dt (R + dt K v + f_ext)
//   A   = M - dt^2 K                      (C = 0: TIMESTEPPER.cpp:657)
//   LHS = S A S + (I - S),  rhs = S b     (S = 0 blocks at pinned vertices)
// solved by PCG from y = 0 with the stopping rule of Eigen's
// conjugate_gradient (ConjugateGradient.h:28-90).
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

constexpr int kLanes = 8;        // threads per vertex row in the SpMV
constexpr int kSpmvThreads = 256;

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Fixed-order sum over the CTA; result valid in thread 0.  nthreads multiple of 32.
template <int NT>
__device__ __forceinline__ double block_sum(double v, double* sh) {
  v = warp_sum(v);
  const int w = threadIdx.x / 32, l = threadIdx.x % 32;
  if (l == 0) sh[w] = v;
  __syncthreads();
  double s = 0;
  if (threadIdx.x == 0) {
#pragma unroll
    for (int i = 0; i < NT / 32; i++) s += sh[i];
  }
  __syncthreads();
  return s;
}

// After a CTA wrote its partial(s): returns true in the CTA that finishes the
// scene's reduction (ticket == ntiles - 1).  The ticket is reset for reuse.
__device__ __forceinline__ bool last_tile(unsigned* ticket, int ntiles, int* flag) {
  __threadfence();
  if (threadIdx.x == 0) {
    const unsigned t = atomicAdd(ticket, 1u);
    *flag = (t == (unsigned)(ntiles - 1));
    if (*flag) *ticket = 0u;
  }
  __syncthreads();
  const bool last = *flag != 0;
  if (last) __threadfence();
  return last;
}

// Sum partial[tile0 .. tile0+n) (stride `stride`, component `comp`) in a fixed
// order with all threads of the CTA; valid in thread 0.
template <int NT>
__device__ __forceinline__ double sum_partials(const double* partial, int tile0, int n, int stride, int comp,
                                               double* sh) {
  double s = 0;
  for (int i = threadIdx.x; i < n; i += NT) s += __ldcg(&partial[(size_t)(tile0 + i) * stride + comp]);
  return block_sum<NT>(s, sh);
}

// x[pinned] = pin target at the start of a step
// (applyKinematicConstraints, TIMESTEPPER.cpp:105-122).
__global__ void k_begin_step(DeviceBatch b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv || b.freeMask[u]) return;
#pragma unroll
  for (int i = 0; i < 3; i++) b.x[3 * u + i] = b.pinTarget[3 * u + i];
}

// One thread per (block, entry): LHS block = S(M - dt^2 K)S + (I - S), with
// K's block the ascending-tet sum of its element contributions
// (TET_MESH_FASTER.cpp:113-131 gathers the same entries per non-zero).
__global__ void k_assemble(DeviceBatch b) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g >= 9L * b.nblocks) return;
  const int blk = (int)(g / 9), e = (int)(g % 9);
  const int r = e / 3, c = e % 3;
  double sum = 0.0;
  const int k0 = b.blkptr[blk], k1 = b.blkptr[blk + 1];
  for (int k = k0; k < k1; k++) {
    const int src = b.blksrc[k];
    const int t = src >> 4, ea = (src >> 2) & 3, eb = src & 3;
    const double* H = b.elemH + (size_t)kElemHess * t;
    sum += (ea <= eb) ? H[9 * upper_block(ea, eb) + 3 * r + c] : H[9 * upper_block(eb, ea) + 3 * c + r];
  }
  const int u = b.blkRow[blk], w = b.cols[blk];
  const double dt = b.scenes[b.vertexScene[u]].dt;
  const bool fu = b.freeMask[u] != 0, fw = b.freeMask[w] != 0;
  double val = (fu && fw) ? -(dt * dt) * sum : 0.0;
  if (u == w && r == c) val += fu ? b.mass[u] : 1.0;
  b.lhs[9 * (size_t)blk + e] = val;
}

// Raw K blocks (column major) and R: the reference's stiffness and force
// outputs (TET_MESH_FASTER.cpp:89-133, TET_MESH.cpp:736-770) for inspection.
__global__ void k_assemble_raw(DeviceBatch b, double* K, double* R) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < 9L * b.nblocks) {
    const int blk = (int)(g / 9), e = (int)(g % 9);
    const int r = e / 3, c = e % 3;
    double sum = 0.0;
    for (int k = b.blkptr[blk]; k < b.blkptr[blk + 1]; k++) {
      const int src = b.blksrc[k];
      const int t = src >> 4, ea = (src >> 2) & 3, eb = src & 3;
      const double* H = b.elemH + (size_t)kElemHess * t;
      sum += (ea <= eb) ? H[9 * upper_block(ea, eb) + 3 * r + c] : H[9 * upper_block(eb, ea) + 3 * c + r];
    }
    K[9 * (size_t)blk + r + 3 * c] = sum;
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
__global__ void k_diag_inverse(DeviceBatch b, int precond) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv) return;
  int k = b.rowptr[u];
  while (b.cols[k] != u) k++;
  const double* D = b.lhs + 9 * (size_t)k;
  double* M = b.minv + 9 * (size_t)u;
  if (precond == 1) {
    const double c00 = D[4] * D[8] - D[5] * D[7];
    const double c01 = D[5] * D[6] - D[3] * D[8];
    const double c02 = D[3] * D[7] - D[4] * D[6];
    const double det = D[0] * c00 + D[1] * c01 + D[2] * c02;
    const double id = 1.0 / det;
    M[0] = c00 * id;
    M[1] = (D[2] * D[7] - D[1] * D[8]) * id;
    M[2] = (D[1] * D[5] - D[2] * D[4]) * id;
    M[3] = c01 * id;
    M[4] = (D[0] * D[8] - D[2] * D[6]) * id;
    M[5] = (D[2] * D[3] - D[0] * D[5]) * id;
    M[6] = c02 * id;
    M[7] = (D[1] * D[6] - D[0] * D[7]) * id;
    M[8] = (D[0] * D[4] - D[1] * D[3]) * id;
  } else {
#pragma unroll
    for (int i = 0; i < 9; i++) M[i] = 0.0;
#pragma unroll
    for (int i = 0; i < 3; i++) M[4 * i] = D[4 * i] != 0.0 ? 1.0 / D[4 * i] : 1.0;
  }
}

// rhs = S dt (sum_e g_e + f_ext) per vertex (element g already carries
// dt (f + dt He v)), then PCG start: y = 0, r = rhs, z = Minv r, p = 0.
// Per-scene: rhsNorm2, threshold and the early exits of conjugate_gradient.
__global__ void __launch_bounds__(kTileV) k_pcg_init(DeviceBatch b) {
  __shared__ double sh[kTileV / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  const int u = b.tileV0[tile] + threadIdx.x;
  double rr = 0, rz = 0;
  if (u < b.tileV1[tile]) {
    const double dt = b.scenes[s].dt;
    double acc[3] = {0.0, 0.0, 0.0};
    for (int k = b.vtxptr[u]; k < b.vtxptr[u + 1]; k++) {
      const int inc = b.vtxinc[k];
      const double* g = b.elemG + 12 * (size_t)(inc >> 2) + 3 * (inc & 3);
#pragma unroll
      for (int i = 0; i < 3; i++) acc[i] += g[i];
    }
    const bool fu = b.freeMask[u] != 0;
    double r3[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      r3[i] = fu ? acc[i] + dt * b.fext[3 * u + i] : 0.0;
      b.rhs[3 * u + i] = r3[i];
      b.r[3 * u + i] = r3[i];
      b.y[3 * u + i] = 0.0;
      b.p0[3 * u + i] = 0.0;
      b.p1[3 * u + i] = 0.0;
    }
    const double* M = b.minv + 9 * (size_t)u;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double zi = M[3 * i] * r3[0] + M[3 * i + 1] * r3[1] + M[3 * i + 2] * r3[2];
      b.z[3 * u + i] = zi;
      rr += r3[i] * r3[i];
      rz += r3[i] * zi;
    }
  }
  const double trr = block_sum<kTileV>(rr, sh);
  const double trz = block_sum<kTileV>(rz, sh);
  if (threadIdx.x == 0) {
    b.partial[2 * tile] = trr;
    b.partial[2 * tile + 1] = trz;
  }
  SolveState& st = b.solve[s];
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketB, sp.ntiles, &flag)) return;
  const double srr = sum_partials<kTileV>(b.partial, sp.tile0, sp.ntiles, 2, 0, sh);
  const double srz = sum_partials<kTileV>(b.partial, sp.tile0, sp.ntiles, 2, 1, sh);
  if (threadIdx.x == 0) {
    st.rhsNorm2 = srr;
    st.threshold = fmax(st.tol * st.tol * srr, DBL_MIN);
    st.rr = srr;
    st.rz = srz;
    st.beta = 0.0;
    st.iters = 0;
    st.converged = 0;
    st.done = 0;
    if (srr == 0.0 || srr < st.threshold) {
      st.done = 1;
      st.converged = 1;
      atomicSub(b.active, 1);
    }
  }
}

// Ap = LHS p with p = z + beta pOld formed on the fly (own rows written to
// pNew), and the scene's p.Ap -> alpha = rz / p.Ap.
__global__ void __launch_bounds__(kSpmvThreads) k_spmv(DeviceBatch b, const double* __restrict__ pOld,
                                                       double* __restrict__ pNew) {
  __shared__ double sh[kSpmvThreads / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  SolveState& st = b.solve[s];
  if (st.done) return;
  const double beta = st.beta;
  const int v0 = b.tileV0[tile], v1 = b.tileV1[tile];
  const int lane = threadIdx.x % kLanes;
  const double* __restrict__ z = b.z;
  double pap = 0.0;
  constexpr int kRowsPerPass = kSpmvThreads / kLanes;
  const int passes = (v1 - v0 + kRowsPerPass - 1) / kRowsPerPass;  // uniform: shuffles need every lane
  for (int pass = 0; pass < passes; pass++) {
    const int u = v0 + pass * kRowsPerPass + threadIdx.x / kLanes;
    const bool valid = u < v1;
    double a0 = 0.0, a1 = 0.0, a2 = 0.0;
    const int k1 = valid ? b.rowptr[u + 1] : 0;
    for (int k = valid ? b.rowptr[u] + lane : 0; k < k1; k += kLanes) {
      const int w = b.cols[k];
      const double q0 = z[3 * w] + beta * pOld[3 * w];
      const double q1 = z[3 * w + 1] + beta * pOld[3 * w + 1];
      const double q2 = z[3 * w + 2] + beta * pOld[3 * w + 2];
      const double* B = b.lhs + 9 * (size_t)k;
      a0 += B[0] * q0 + B[1] * q1 + B[2] * q2;
      a1 += B[3] * q0 + B[4] * q1 + B[5] * q2;
      a2 += B[6] * q0 + B[7] * q1 + B[8] * q2;
    }
#pragma unroll
    for (int o = kLanes / 2; o > 0; o >>= 1) {
      a0 += __shfl_xor_sync(0xffffffffu, a0, o);
      a1 += __shfl_xor_sync(0xffffffffu, a1, o);
      a2 += __shfl_xor_sync(0xffffffffu, a2, o);
    }
    if (valid && lane == 0) {
      const double p0 = z[3 * u] + beta * pOld[3 * u];
      const double p1 = z[3 * u + 1] + beta * pOld[3 * u + 1];
      const double p2 = z[3 * u + 2] + beta * pOld[3 * u + 2];
      pNew[3 * u] = p0;
      pNew[3 * u + 1] = p1;
      pNew[3 * u + 2] = p2;
      b.Ap[3 * u] = a0;
      b.Ap[3 * u + 1] = a1;
      b.Ap[3 * u + 2] = a2;
      pap += p0 * a0 + p1 * a1 + p2 * a2;
    }
  }
  const double tp = block_sum<kSpmvThreads>(pap, sh);
  if (threadIdx.x == 0) b.partial[2 * tile] = tp;
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketA, sp.ntiles, &flag)) return;
  const double spap = sum_partials<kSpmvThreads>(b.partial, sp.tile0, sp.ntiles, 2, 0, sh);
  if (threadIdx.x == 0) st.alpha = st.rz / spap;
}

// y += alpha p; r -= alpha Ap; z = Minv r; then the residual test and beta
// (ConjugateGradient.h:69-86).
__global__ void __launch_bounds__(kTileV) k_update(DeviceBatch b, const double* __restrict__ p) {
  __shared__ double sh[kTileV / 32];
  __shared__ int flag;
  const int tile = blockIdx.x;
  const int s = b.tileScene[tile];
  SolveState& st = b.solve[s];
  if (st.done) return;
  const double alpha = st.alpha;
  const int u = b.tileV0[tile] + threadIdx.x;
  double rr = 0, rz = 0;
  if (u < b.tileV1[tile]) {
    double r3[3];
#pragma unroll
    for (int i = 0; i < 3; i++) {
      b.y[3 * u + i] += alpha * p[3 * u + i];
      r3[i] = b.r[3 * u + i] - alpha * b.Ap[3 * u + i];
      b.r[3 * u + i] = r3[i];
      rr += r3[i] * r3[i];
    }
    const double* M = b.minv + 9 * (size_t)u;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const double zi = M[3 * i] * r3[0] + M[3 * i + 1] * r3[1] + M[3 * i + 2] * r3[2];
      b.z[3 * u + i] = zi;
      rz += r3[i] * zi;
    }
  }
  const double trr = block_sum<kTileV>(rr, sh);
  const double trz = block_sum<kTileV>(rz, sh);
  if (threadIdx.x == 0) {
    b.partial[2 * tile] = trr;
    b.partial[2 * tile + 1] = trz;
  }
  const SceneParams& sp = b.scenes[s];
  if (!last_tile(&st.ticketB, sp.ntiles, &flag)) return;
  const double srr = sum_partials<kTileV>(b.partial, sp.tile0, sp.ntiles, 2, 0, sh);
  const double srz = sum_partials<kTileV>(b.partial, sp.tile0, sp.ntiles, 2, 1, sh);
  if (threadIdx.x == 0) {
    st.rr = srr;
    if (srr < st.threshold) {
      st.done = 1;
      st.converged = 1;
      atomicSub(b.active, 1);
    } else if (!(srr == srr) || !(srz == srz)) {
      st.done = 1;  // non-finite: stop, the host reports HOBAK_ERR_NAN
      st.converged = -1;
      atomicSub(b.active, 1);
    } else {
      st.beta = srz / st.rz;
      st.rz = srz;
      st.iters += 1;
      if (st.iters >= st.maxit) {
        st.done = 1;
        atomicSub(b.active, 1);
      }
    }
  }
}

// v += y; x += dt v; v = S v (BACKWARD_EULER_VELOCITY.cpp:191-201).
__global__ void k_finish_step(DeviceBatch b) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= b.nv) return;
  const double dt = b.scenes[b.vertexScene[u]].dt;
  const bool fu = b.freeMask[u] != 0;
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

void launch_assemble(const DeviceBatch& b, cudaStream_t s) {
  const long n = 9L * b.nblocks;
  k_assemble<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b);
}

void launch_assemble_raw(const DeviceBatch& b, double* K, double* R, cudaStream_t s) {
  const long n = std::max(9L * b.nblocks, 3L * b.nv);
  k_assemble_raw<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(b, K, R);
}

void launch_diag_inverse(const DeviceBatch& b, int precond, cudaStream_t s) {
  k_diag_inverse<<<(b.nv + 255) / 256, 256, 0, s>>>(b, precond);
}

void launch_pcg_init(const DeviceBatch& b, cudaStream_t s) { k_pcg_init<<<b.ntiles, kTileV, 0, s>>>(b); }

void launch_spmv(const DeviceBatch& b, const double* pOld, double* pNew, cudaStream_t s) {
  k_spmv<<<b.ntiles, kSpmvThreads, 0, s>>>(b, pOld, pNew);
}

void launch_update(const DeviceBatch& b, const double* p, cudaStream_t s) {
  k_update<<<b.ntiles, kTileV, 0, s>>>(b, p);
}

void launch_pcg_iteration(const DeviceBatch& b, const double* pOld, double* pNew, cudaStream_t s) {
  launch_spmv(b, pOld, pNew, s);
  launch_update(b, pNew, s);
}

void launch_finish_step(const DeviceBatch& b, cudaStream_t s) {
  k_finish_step<<<(b.nv + 255) / 256, 256, 0, s>>>(b);
}

}  // namespace hobak
