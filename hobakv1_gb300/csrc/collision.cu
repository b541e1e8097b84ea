// Vertex-face self collisions on the GPU.
//
// Per step, for the scenes that have them on:
//   1. inverted vertices: any incident tet with det F <= 0
//      (TET_MESH::computeInvertedVertices, TET_MESH.cpp:2450-2475);
//   2. broad phase: a spatial hash of the surface triangles' AABBs inflated by
//      the collision distance; the cell size is the scene's largest inflated
//      triangle extent, so each triangle covers at most 2x2x2 cells and a
//      vertex only has to look in its own cell.  It replaces the AABB tree
//      (AABB_TREE.cpp:563-578); being conservative, it leaves the narrow
//      phase's answer unchanged;
//   3. narrow phase per surface vertex, exactly the tests of
//      TET_MESH_FASTER::computeVertexFaceCollisions (TET_MESH_FASTER.cpp:248-334):
//      skip inverted vertices, degenerate triangles (relative area < 1e-4,
//      TET_MESH.cpp:2421-2445), all-inverted faces and the vertex's own
//      triangles; accept when pointTriangleDistance < eps (TET_MESH.cpp:1322-1388)
//      and the vertex projects inside the triangle (1296-1317) or lies inside
//      its collision cell (1396-1437);
//   4. collision tets (v, f2, f1, f0) weighted by rest face area + rest vertex
//      one-ring area (TET_MESH.cpp:1785-1826), VERTEX_FACE_SQRT_COLLISION force
//      and clamped Hessian (VERTEX_FACE_SQRT_COLLISION.cpp:140-219).  The
//      Hessian is 2 mu (c c^T) (x) (k1 t t^T + k2 I) with c = (1, -bary):
//      its eigenvalues are 2 mu |c|^2 along t and 2 mu |c|^2 k2 across it, so
//      the clamp of MATRIX_UTIL.cpp:116-127 is exact in closed form:
//      H+ = 2 mu (c c^T) (x) (that + max(k2, 0)(I - that that^T)).
//   5. per-vertex incidence lists (sorted by pair) for the gathers in the rhs,
//      the SpMV and the preconditioner.
#include <cfloat>

#include "collision.cuh"
#include <algorithm>
#include "kernels.cuh"

namespace hobak {

namespace {

struct D3 {
  double x, y, z;
};
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator*(double s, D3 a) { return {s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ double dot(D3 a, D3 b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
__device__ __forceinline__ D3 cross(D3 a, D3 b) {
  return {a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x};
}
__device__ __forceinline__ double norm(D3 a) { return sqrt(dot(a, a)); }
__device__ __forceinline__ D3 unit(D3 a) { return (1.0 / norm(a)) * a; }

// NEWMARK: beta G sum_b c_b (a3 (x_b - x_old_b) + a4 v_old_b + a5 a_old_b),
// the pair's share of C times the Newmark velocity term (C = beta H_coll,
// NEWMARK.cpp:244-255; G is the pair's 3x3 factor of H_coll, column major).
__device__ __forceinline__ void newmark_coll_term(const DeviceBatch& b, int s, const int* id, const double* cvec,
                                                  const double* G, double beta, double* out) {
  const double* nm = b.scenes[s].nm;
  double z[3] = {0.0, 0.0, 0.0};
  for (int q = 0; q < 4; q++)
    for (int k = 0; k < 3; k++) {
      const size_t i = 3 * (size_t)id[q] + k;
      z[k] += cvec[q] * (nm[3] * (b.x[i] - b.xOld[i]) + nm[4] * b.vOld[i] + nm[5] * b.aOld[i]);
    }
  for (int r = 0; r < 3; r++) out[r] = beta * (G[r] * z[0] + G[r + 3] * z[1] + G[r + 6] * z[2]);
}

__device__ __forceinline__ D3 pos(const DeviceBatch& b, int v) {
  return {b.rest[3 * v] + b.x[3 * v], b.rest[3 * v + 1] + b.x[3 * v + 1], b.rest[3 * v + 2] + b.x[3 * v + 2]};
}

__device__ __forceinline__ unsigned hash_cell(int scene, int cx, int cy, int cz, int mask) {
  unsigned h = (unsigned)cx * 73856093u ^ (unsigned)cy * 19349663u ^ (unsigned)cz * 83492791u ^
               (unsigned)scene * 2654435761u;
  return h & (unsigned)mask;
}

// Largest inflated triangle extent, widened by 1e-6 so rounding can never make
// a triangle span a third cell along an axis.
__device__ __forceinline__ double cell_size(const DeviceCollisions& c, int scene) {
  return fmax((double)__uint_as_float(c.cellBits[scene]), 1e-12) * (1.0 + 1e-6);
}

// ---- device-wide exclusive scan of int counts (in place, n + 1 outputs) ----
constexpr int kScanThreads = 1024;

__global__ void k_scan_blocks(int* data, int n, int* blockSums) {
  __shared__ int sh[kScanThreads];
  const int i = blockIdx.x * kScanThreads + threadIdx.x;
  const int v = i < n ? data[i] : 0;
  sh[threadIdx.x] = v;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  if (i < n) data[i] = sh[threadIdx.x] - v;  // exclusive within the block
  if (threadIdx.x == kScanThreads - 1) blockSums[blockIdx.x] = sh[threadIdx.x];
}

// One CTA scans the block sums (serially per thread chunk); writes data[n] = total.
__global__ void k_scan_sums(int* blockSums, int nblocks, int* data, int n) {
  __shared__ int sh[kScanThreads];
  const int per = (nblocks + kScanThreads - 1) / kScanThreads;
  const int b0 = threadIdx.x * per;
  int s = 0;
  for (int k = 0; k < per && b0 + k < nblocks; k++) s += blockSums[b0 + k];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < kScanThreads; o <<= 1) {
    const int t = threadIdx.x >= o ? sh[threadIdx.x - o] : 0;
    __syncthreads();
    sh[threadIdx.x] += t;
    __syncthreads();
  }
  int run = sh[threadIdx.x] - s;
  for (int k = 0; k < per && b0 + k < nblocks; k++) {
    const int v = blockSums[b0 + k];
    blockSums[b0 + k] = run;
    run += v;
  }
  if (threadIdx.x == kScanThreads - 1) data[n] = sh[threadIdx.x];
}

__global__ void k_scan_add(int* data, int n, const int* blockSums) {
  const int i = blockIdx.x * kScanThreads + threadIdx.x;
  if (i < n) data[i] += blockSums[blockIdx.x];
}

// data[0..n) counts -> exclusive offsets, data[n] = total.  n <= 1024^2 * 1024.
void scan_counts(int* data, int n, int* tmp, cudaStream_t s) {
  const int nb = (n + kScanThreads - 1) / kScanThreads;
  k_scan_blocks<<<nb, kScanThreads, 0, s>>>(data, n, tmp);
  k_scan_sums<<<1, kScanThreads, 0, s>>>(tmp, nb, data, n);
  k_scan_add<<<nb, kScanThreads, 0, s>>>(data, n, tmp);
}

// ---- 1. inverted vertices ----
__global__ void k_mark_inverted(DeviceBatch b, DeviceCollisions c) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= b.nt) return;
  const int s = b.tetScene[t];
  if (!c.scenes[s].vfOn) return;
  const int4 tv = b.tets[t];
  const int vid[4] = {tv.x, tv.y, tv.z, tv.w};
  const D3 x0 = pos(b, vid[0]);
  double Ds[9], F[9];
  for (int a = 0; a < 3; a++) {
    const D3 d = pos(b, vid[a + 1]) - x0;
    Ds[3 * a] = d.x;
    Ds[3 * a + 1] = d.y;
    Ds[3 * a + 2] = d.z;
  }
  const double* Di = b.DmInv + 9 * (size_t)t;
  for (int j = 0; j < 3; j++)
    for (int i = 0; i < 3; i++) F[i + 3 * j] = Ds[i] * Di[3 * j] + Ds[i + 3] * Di[1 + 3 * j] + Ds[i + 6] * Di[2 + 3 * j];
  const double det = F[0] * (F[4] * F[8] - F[7] * F[5]) - F[3] * (F[1] * F[8] - F[7] * F[2]) +
                     F[6] * (F[1] * F[5] - F[4] * F[2]);
  if (det > 0.0) return;
  for (int a = 0; a < 4; a++) c.vInverted[vid[a]] = 1;  // every writer stores 1
}

// ---- 2. triangle flags and cell size ----
__global__ void k_tri_prepare(DeviceBatch b, DeviceCollisions c) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= c.ntri) return;
  const int s = c.triScene[f];
  const CollisionScene& cs = c.scenes[s];
  if (!cs.vfOn) return;
  const int v0 = c.tri[3 * f], v1 = c.tri[3 * f + 1], v2 = c.tri[3 * f + 2];
  const D3 a = pos(b, v0), bb = pos(b, v1), cc = pos(b, v2);
  const double area = 0.5 * norm(cross(bb - a, cc - a));
  const bool degenerate = area / c.triArea[f] < 1e-4;
  const bool allInv = c.vInverted[v0] && c.vInverted[v1] && c.vInverted[v2];
  c.triSkip[f] = (degenerate || allInv) ? 1 : 0;
  const double ext = fmax(fmax(fmax(fmax(a.x, bb.x), cc.x) - fmin(fmin(a.x, bb.x), cc.x),
                               fmax(fmax(a.y, bb.y), cc.y) - fmin(fmin(a.y, bb.y), cc.y)),
                          fmax(fmax(a.z, bb.z), cc.z) - fmin(fmin(a.z, bb.z), cc.z)) +
                     2.0 * cs.eps;
  // positive floats order like their bit patterns; round up so the cell covers ext
  atomicMax(&c.cellBits[s], __float_as_uint(__double2float_ru(ext)));
}

template <bool FILL>
__global__ void k_tri_bucket(DeviceBatch b, DeviceCollisions c) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= c.ntri) return;
  const int s = c.triScene[f];
  const CollisionScene& cs = c.scenes[s];
  if (!cs.vfOn) return;
  const D3 a = pos(b, c.tri[3 * f]), bb = pos(b, c.tri[3 * f + 1]), cc = pos(b, c.tri[3 * f + 2]);
  const double h = cell_size(c, s), e = cs.eps;
  const int x0 = (int)floor((fmin(fmin(a.x, bb.x), cc.x) - e) / h), x1 = (int)floor((fmax(fmax(a.x, bb.x), cc.x) + e) / h);
  const int y0 = (int)floor((fmin(fmin(a.y, bb.y), cc.y) - e) / h), y1 = (int)floor((fmax(fmax(a.y, bb.y), cc.y) + e) / h);
  const int z0 = (int)floor((fmin(fmin(a.z, bb.z), cc.z) - e) / h), z1 = (int)floor((fmax(fmax(a.z, bb.z), cc.z) + e) / h);
  const int mask = c.hashSize - 1;
  // at most 2 cells per axis by the choice of h; the loops are bounded anyway
  for (int ix = x0; ix <= x1 && ix <= x0 + 1; ix++)
    for (int iy = y0; iy <= y1 && iy <= y0 + 1; iy++)
      for (int iz = z0; iz <= z1 && iz <= z0 + 1; iz++) {
        const unsigned bk = hash_cell(s, ix, iy, iz, mask);
        if (!FILL) {
          atomicAdd(&c.bucketCount[bk], 1);
        } else {
          const int p = c.bucketCount[bk] + atomicAdd(&c.bucketCursor[bk], 1);
          c.entryTri[p] = f;
        }
      }
}

// ---- 3. narrow phase per surface vertex ----
__device__ bool projects_inside(D3 v0, D3 v1, D3 v2, D3 v) {
  const D3 n = cross(v1 - v0, v2 - v0);
  const double nn = dot(n, n);
  const double b0 = dot(n, cross(v2 - v1, v - v1)) / nn;
  const double b1 = dot(n, cross(v0 - v2, v - v2)) / nn;
  const double b2 = dot(n, cross(v1 - v0, v - v0)) / nn;
  return fabs(b0) + fabs(b1) + fabs(b2) - 1.0 < 1e-8;
}

__device__ double point_triangle_distance(D3 v0, D3 v1, D3 v2, D3 v) {
  const D3 e1 = v1 - v0, e2 = v2 - v0;
  const D3 n = cross(e1, e2);
  if (projects_inside(v0, v1, v2, v)) return fabs(dot((1.0 / norm(n)) * n, v - v0));
  const D3 e3 = v2 - v1, ev = v - v0, ev3 = v - v1;
  const double big = (double)FLT_MAX;
  double d0 = big, d1 = big, d2 = big;
  const double l1 = norm(e1), l2 = norm(e2), l3 = norm(e3);
  const D3 h1 = (1.0 / l1) * e1, h2 = (1.0 / l2) * e2, h3 = (1.0 / l3) * e3;
  const double p1 = dot(h1, ev), p2 = dot(h2, ev), p3 = dot(h3, ev3);
  if (p1 > 0.0 && p1 < l1) d0 = norm(v - (v0 + p1 * h1));
  if (p2 > 0.0 && p2 < l2) d1 = norm(v - (v0 + p2 * h2));
  if (p3 > 0.0 && p3 < l3) d2 = norm(v - (v1 + p3 * h3));
  const double vmin = fmin(norm(v - v0), fmin(norm(v - v1), norm(v - v2)));
  const double emin = fmin(d0, fmin(d1, d2));
  return vmin < emin ? vmin : emin;
}

__device__ bool inside_collision_cell(const DeviceBatch& b, const DeviceCollisions& c, int f, D3 p) {
  const D3 vv[3] = {pos(b, c.tri[3 * f]), pos(b, c.tri[3 * f + 1]), pos(b, c.tri[3 * f + 2])};
  const D3 n = unit(cross(vv[1] - vv[0], vv[2] - vv[0]));
  for (int k = 0; k < 3; k++) {
    const int g = c.triNbr[3 * f + k];
    if (g < 0) return false;
    const D3 na = pos(b, c.tri[3 * g]), nb = pos(b, c.tri[3 * g + 1]), nc = pos(b, c.tri[3 * g + 2]);
    const D3 nn = unit(cross(nb - na, nc - na));
    const D3 ne = unit(nn + n);
    const D3 neb = unit(cross(ne, vv[(k + 1) % 3] - vv[k]));
    if (dot(neb, p - vv[k]) < 0.0) return false;
  }
  return true;
}

__global__ void k_vf_query(DeviceBatch b, DeviceCollisions c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nsv) return;
  c.svCount[i] = 0;
  const int s = c.svScene[i];
  const CollisionScene& cs = c.scenes[s];
  const int v = c.sv[i];
  if (!cs.vfOn || c.vInverted[v]) return;
  const D3 p = pos(b, v);
  const double h = cell_size(c, s);
  const unsigned bk = hash_cell(s, (int)floor(p.x / h), (int)floor(p.y / h), (int)floor(p.z / h), c.hashSize - 1);
  int found[kMaxPairsPerVertex];
  int n = 0;
  bool over = false;
  for (int k = c.bucketCount[bk]; k < c.bucketCount[bk + 1]; k++) {
    const int f = c.entryTri[k];
    if (c.triScene[f] != s || c.triSkip[f]) continue;
    const int t0 = c.tri[3 * f], t1 = c.tri[3 * f + 1], t2 = c.tri[3 * f + 2];
    if (t0 == v || t1 == v || t2 == v) continue;
    bool dup = false;
    for (int j = 0; j < n; j++) dup |= (found[j] == f);
    if (dup) continue;
    const D3 a = pos(b, t0), bb = pos(b, t1), cc = pos(b, t2);
    if (!(point_triangle_distance(a, bb, cc, p) < cs.eps)) continue;
    if (!projects_inside(a, bb, cc, p) && !inside_collision_cell(b, c, f, p)) continue;
    if (n < kMaxPairsPerVertex) {
      // insertion keeps the list ascending by triangle id
      int j = n++;
      while (j > 0 && found[j - 1] > f) {
        found[j] = found[j - 1];
        j--;
      }
      found[j] = f;
    } else {
      over = true;
    }
  }
  if (over) atomicExch(c.overflow, 1);
  for (int j = 0; j < n; j++) c.svCand[kMaxPairsPerVertex * (size_t)i + j] = found[j];
  c.svCount[i] = n;
}

// ---- 4. collision tets, forces and clamped Hessians ----
__device__ void vf_barycentric(const D3 v[4], double bary[3]) {
  const D3 n = cross(v[2] - v[1], v[3] - v[1]);
  const D3 nh = unit(n);
  const D3 p = v[0] - dot(nh, v[0] - v[1]) * nh;
  const double nn = dot(n, n);
  bary[0] = dot(n, cross(v[3] - v[2], p - v[2])) / nn;
  bary[1] = dot(n, cross(v[1] - v[3], p - v[3])) / nn;
  bary[2] = dot(n, cross(v[2] - v[1], p - v[1])) / nn;
  if (bary[0] >= 0.0 && bary[1] >= 0.0 && bary[2] >= 0.0) return;
  // closest edge (COLLISION_UTIL.cpp:356-502)
  auto lineDist = [](D3 p0, D3 p1, D3 p2) {
    const D3 e0 = p0 - p1, e = p2 - p1;
    const double l = norm(e);
    const double proj = dot(e0, (1.0 / l) * e);
    if (proj > 0.0 && proj < l) return norm(e0 - proj * ((1.0 / l) * e));
    const double d1 = norm(p0 - p1), d2 = norm(p0 - p2);
    return d1 < d2 ? d1 : d2;
  };
  auto lerp = [](D3 p0, D3 p1, D3 p2, double& l0, double& l1) {
    const D3 e0 = p0 - p1, e = p2 - p1;
    const double l = norm(e);
    const double proj = dot(e0, (1.0 / l) * e);
    if (proj < 0.0) { l0 = 1.0; l1 = 0.0; return; }
    if (proj >= l) { l0 = 0.0; l1 = 1.0; return; }
    const double r = proj / l;
    l0 = 1.0 - r;
    l1 = r;
  };
  const double d12 = lineDist(v[0], v[1], v[2]), d23 = lineDist(v[0], v[2], v[3]), d31 = lineDist(v[0], v[3], v[1]);
  double l0, l1;
  if (d12 <= d23 && d12 <= d31) {
    lerp(v[0], v[1], v[2], l0, l1);
    bary[0] = l0; bary[1] = l1; bary[2] = 0.0;
  } else if (d23 <= d12 && d23 <= d31) {
    lerp(v[0], v[2], v[3], l0, l1);
    bary[0] = 0.0; bary[1] = l0; bary[2] = l1;
  } else {
    lerp(v[0], v[3], v[1], l0, l1);
    bary[0] = l1; bary[1] = 0.0; bary[2] = l0;
  }
}

__global__ void k_vf_pairs(DeviceBatch b, DeviceCollisions c) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= c.nsv) return;
  const int n = c.svCount[i + 1] - c.svCount[i];
  if (n == 0) return;
  const int s = c.svScene[i];
  const CollisionScene& cs = c.scenes[s];
  const double dt = b.scenes[s].dt;
  const int v = c.sv[i];
  for (int j = 0; j < n; j++) {
    const int pidx = c.svCount[i] + j;
    if (pidx >= c.pairCap) {
      atomicExch(c.overflow, 1);
      return;
    }
    const int f = c.svCand[kMaxPairsPerVertex * (size_t)i + j];
    const int4 ct = make_int4(v, c.tri[3 * f + 2], c.tri[3 * f + 1], c.tri[3 * f]);
    c.pairTet[pidx] = ct;
    const double w = c.triArea[f] + c.svArea[i];
    const int id[4] = {ct.x, ct.y, ct.z, ct.w};
    D3 x[4];
    for (int a = 0; a < 4; a++) x[a] = pos(b, id[a]);
    double bary[3];
    vf_barycentric(x, bary);
    const D3 e0 = x[3] - x[2], e1 = x[0] - x[2], e2 = x[1] - x[2];
    const bool reversal = dot(unit(cross(e2, e0)), e1) < 0.0;
    const D3 t = x[0] - (bary[0] * x[1] + bary[1] * x[2] + bary[2] * x[3]);
    const double tt = dot(t, t), tm = sqrt(tt);
    const double spring = reversal ? tm + cs.eps : tm - cs.eps;
    const double cvec[4] = {1.0, -bary[0], -bary[1], -bary[2]};
    double* C = c.pairC + 4 * (size_t)pidx;
    double* G = c.pairG + 9 * (size_t)pidx;
    double* R = c.pairRhs + 12 * (size_t)pidx;
    for (int a = 0; a < 4; a++) C[a] = cvec[a];
    double* Fo = c.pairF + 12 * (size_t)pidx;
    if (fabs(tm) <= 1e-8 || fabs(tt) < 1e-8) {  // VERTEX_FACE_SQRT_COLLISION.cpp:158,206
      for (int k = 0; k < 9; k++) G[k] = 0.0;
      for (int k = 0; k < 12; k++) R[k] = Fo[k] = 0.0;
      continue;
    }
    // force -w grad = -w 2 mu spring / tm (c (x) t)
    const double fs = -w * 2.0 * cs.mu * spring / tm;
    // clamped Hessian factor: -w 2 mu (that that^T + max(spring/tm, 0)(I - that that^T))
    const D3 th = (1.0 / tm) * t;
    const double k2 = fmax(spring / tm, 0.0);
    const double th3[3] = {th.x, th.y, th.z};
    const double gs = -w * 2.0 * cs.mu;
    for (int r = 0; r < 3; r++)
      for (int q = 0; q < 3; q++) G[r + 3 * q] = gs * ((1.0 - k2) * th3[r] * th3[q] + (r == q ? k2 : 0.0));
    // H v = (c c^T) (x) G v: zv = sum_b c_b v_b, (H v)_a = c_a G zv
    double zv[3] = {0, 0, 0};
    for (int bb2 = 0; bb2 < 4; bb2++)
      for (int k = 0; k < 3; k++) zv[k] += cvec[bb2] * b.v[3 * id[bb2] + k];
    double Gz[3];
    for (int r = 0; r < 3; r++) Gz[r] = G[r] * zv[0] + G[r + 3] * zv[1] + G[r + 6] * zv[2];
    const double tv[3] = {t.x, t.y, t.z};
    // right-hand side: dt (f + dt H v) for the velocity integrator; the
    // position integrator's b takes the force alone (collisionC and K stay
    // out of it, BACKWARD_EULER_POSITION.cpp:196-203); NEWMARK's b subtracts
    // f + beta H (a3 (x - x_old) + a4 v_old + a5 a_old) (C = beta H_coll,
    // NEWMARK.cpp:244-255)
    const int integ = b.scenes[s].integrator;
    double Gn[3] = {0.0, 0.0, 0.0};
    if (integ == kIntegratorNewmark) newmark_coll_term(b, s, id, cvec, G, cs.beta, Gn);
    for (int a = 0; a < 4; a++)
      for (int k = 0; k < 3; k++) {
        Fo[3 * a + k] = fs * cvec[a] * tv[k];
        R[3 * a + k] = integ == kIntegratorPosition ? fs * cvec[a] * tv[k]
                       : integ == kIntegratorNewmark ? fs * cvec[a] * tv[k] + cvec[a] * Gn[k]
                                                     : dt * (fs * cvec[a] * tv[k] + dt * cvec[a] * Gz[k]);
      }
  }
}

// ---- 5. per-vertex incidence lists ----
__global__ void k_inc_count(DeviceCollisions c) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = min(*c.npairs, c.pairCap);
  if (g >= 4 * np) return;
  const int4 ct = c.pairTet[g / 4];
  const int slot = g % 4;
  const int v = slot == 0 ? ct.x : slot == 1 ? ct.y : slot == 2 ? ct.z : ct.w;
  atomicAdd(&c.incCount[v], 1);
}

__global__ void k_inc_fill(DeviceCollisions c) {
  const int g = blockIdx.x * blockDim.x + threadIdx.x;
  const int np = min(*c.npairs, c.pairCap);
  if (g >= 4 * np) return;
  const int4 ct = c.pairTet[g / 4];
  const int slot = g % 4;
  const int v = slot == 0 ? ct.x : slot == 1 ? ct.y : slot == 2 ? ct.z : ct.w;
  c.incList[c.incCount[v] + atomicAdd(&c.incCursor[v], 1)] = g;
}

__global__ void k_inc_sort(DeviceCollisions c) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= c.nv) return;
  int* L = c.incList + c.incCount[v];
  const int n = c.incCount[v + 1] - c.incCount[v];
  for (int i = 1; i < n; i++) {
    const int x = L[i];
    int j = i;
    while (j > 0 && L[j - 1] > x) {
      L[j] = L[j - 1];
      j--;
    }
    L[j] = x;
  }
}

__global__ void k_copy_total(const int* src, int* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst = *src;
}

// Collision part of LHS's diagonal, w sum c_a^2 G (w = collision_lhs_scale) over the
// vertex's incidences (free rows only; zero elsewhere), kept in FP64 beside
// the LHS: the preconditioner adds it to the diagonal block, the products
// (collision_row) apply it in FP64, so the mixed path's FP64 residual sees the
// stiff contact block unrounded.
__global__ void k_coll_diag(DeviceBatch b, DeviceCollisions c) {
  const int u = blockIdx.x * blockDim.x + threadIdx.x;
  if (u >= c.nv) return;
  double* out = c.diag + 9 * (size_t)u;
  const int k0 = c.incCount[u], k1 = c.incCount[u + 1];
  if (k0 == k1 || !b.freeMask[u]) {
#pragma unroll
    for (int q = 0; q < 9; q++) out[q] = 0.0;
    return;
  }
  const double scale = collision_lhs_scale(b, b.vertexScene[u]);
  double D[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int k = k0; k < k1; k++) {
    const int e = c.incList[k], p = e >> 2, a = e & 3;
    const double ca = c.pairC[4 * (size_t)p + a];
    for (int q = 0; q < 9; q++) D[q] += scale * ca * ca * c.pairG[9 * (size_t)p + q];
  }
  for (int r = 0; r < 3; r++)
    for (int q = 0; q < 3; q++) out[3 * r + q] = D[r + 3 * q];  // row major like the LHS blocks
}

// ---- 6. edge-edge (TET_MESH_FASTER.cpp:340-500, EDGE_SQRT_COLLISION.cpp) ----
// Closest points of two segments, restating the published routine the
// reference uses (Rhodes, "Fast, Robust Intersection of 3D Line Segments",
// Game Programming Gems II; LINE_INTERSECT.cpp) with its tolerances: 1e-8
// for parallel/degenerate lines, also where its helpers take a squared one.
namespace seg {
constexpr double kTol = 1e-8;
__device__ __forceinline__ bool outside01(double a) { return a < 0.0 || a > 1.0; }
__device__ __forceinline__ double clamp01(double a) { return fmax(0.0, fmin(1.0, a)); }
__device__ void nearest(D3 p, D3 L, D3 q, bool infinite, D3& out, double& param) {
  const double D = dot(L, L);
  if (D < kTol) {
    out = p;
    return;
  }
  param = dot(L, q - p) / D;
  if (!infinite) param = clamp01(param);
  out = p + param * L;
}
__device__ void closest(D3 a1, D3 a2, D3 b1, D3 b2, D3& pa, D3& pb) {
  const D3 La = a2 - a1, Lb = b2 - b1;
  const double L11 = dot(La, La), L22 = dot(Lb, Lb);
  double tmp = 0.0;
  if (L11 < kTol * kTol) {
    pa = a1;
    nearest(b1, Lb, a1, false, pb, tmp);
    return;
  }
  if (L22 < kTol * kTol) {
    pb = b1;
    nearest(a1, La, b1, false, pa, tmp);
    return;
  }
  const D3 AB = b1 - a1;
  const double L12 = -dot(La, Lb);
  const double det = L11 * L22 - L12 * L12;
  if (fabs(det) < kTol) {  // parallel
    double s0 = 0.0, s1 = 0.0;
    D3 scratch;
    nearest(a1, La, b1, true, pa, s0);
    nearest(a1, La, b2, true, scratch, s1);
    if (s0 < 0.0 && s1 < 0.0) {
      pa = a1;
      pb = s0 < s1 ? b2 : b1;
    } else if (s0 > 1.0 && s1 > 1.0) {
      pa = a2;
      pb = s0 < s1 ? b1 : b2;
    } else {
      tmp = 0.5 * (clamp01(s0) + clamp01(s1));
      pa = a1 + tmp * La;
      nearest(b1, Lb, pa, true, pb, tmp);
    }
    return;
  }
  const double ra = dot(La, AB), rb = -dot(Lb, AB);
  double t = (L11 * rb - ra * L12) / det;
  double s = (ra - L12 * t) / L11;
  pa = a1 + s * La;
  pb = b1 + t * Lb;
  if (!(outside01(s) || outside01(t))) return;
  if (outside01(s) && outside01(t)) {
    s = clamp01(s);
    pa = a1 + s * La;
    nearest(b1, Lb, pa, true, pb, t);
    if (outside01(t)) {
      t = clamp01(t);
      pb = b1 + t * Lb;
      nearest(a1, La, pb, false, pa, s);
      nearest(b1, Lb, pa, false, pb, t);
    }
  } else if (outside01(s)) {
    s = clamp01(s);
    pa = a1 + s * La;
    nearest(b1, Lb, pa, false, pb, t);
  } else {
    t = clamp01(t);
    pb = b1 + t * Lb;
    nearest(a1, La, pb, false, pa, s);
  }
}
}  // namespace seg

// faceEdgeIntersection (COLLISION_UTIL.cpp:577-613)
__device__ bool face_edge_cross(D3 a, D3 b, D3 c, D3 e0, D3 e1) {
  const D3 ed = e1 - e0, dir = unit(ed);
  const D3 n = unit(cross(b - a, c - a));
  const double denom = dot(dir, n);
  if (fabs(denom) <= 0.0) return false;
  const double t = dot(a - e0, n) / denom;
  if (t < 0) return false;
  const D3 h = e0 + t * dir;
  if (dot(n, cross(b - a, h - a)) < 0) return false;
  if (dot(n, cross(c - b, h - b)) < 0) return false;
  if (dot(n, cross(a - c, h - c)) < 0) return false;
  return t < norm(ed);
}

// is (u, w) a surface edge of the scene (the one-ring test of
// TET_MESH::computeSurfaceVertexOneRings, TET_MESH.cpp:2145-2155)
__device__ bool surface_edge(const DeviceCollisions& c, const CollisionScene& cs, int u, int w) {
  const int lo = min(u, w), hi = max(u, w);
  int l = cs.e0, r = cs.e0 + cs.ne;
  while (l < r) {
    const int m = (l + r) >> 1;
    const int2 e = c.edge[m];
    if (e.x < lo || (e.x == lo && e.y < hi)) l = m + 1;
    else r = m;
  }
  return l < cs.e0 + cs.ne && c.edge[l].x == lo && c.edge[l].y == hi;
}

__device__ __forceinline__ double ee_cell_size(const DeviceCollisions& c, int scene) {
  return fmax((double)__uint_as_float(c.eeCellBits[scene]), 1e-12) * (1.0 + 1e-6);
}

// the scene's largest eps-inflated edge extent sets its cell size
__global__ void k_edge_prepare(DeviceBatch b, DeviceCollisions c) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= c.nedge) return;
  const int s = c.edgeScene[x];
  const CollisionScene& cs = c.scenes[s];
  if (!cs.eeOn) return;
  const int2 e = c.edge[x];
  const D3 p = pos(b, e.x), q = pos(b, e.y);
  const double ext = fmax(fmax(fabs(p.x - q.x), fabs(p.y - q.y)), fabs(p.z - q.z)) + 2.0 * cs.eps;
  atomicMax(&c.eeCellBits[s], __float_as_uint(__double2float_ru(ext)));
}

// every edge into the cells its eps-inflated box overlaps (<= 2 per axis)
template <bool FILL>
__global__ void k_edge_bucket(DeviceBatch b, DeviceCollisions c) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= c.nedge) return;
  const int s = c.edgeScene[x];
  const CollisionScene& cs = c.scenes[s];
  if (!cs.eeOn) return;
  const int2 e = c.edge[x];
  const D3 p = pos(b, e.x), q = pos(b, e.y);
  const double h = ee_cell_size(c, s), ep = cs.eps;
  const int x0 = (int)floor((fmin(p.x, q.x) - ep) / h), x1 = (int)floor((fmax(p.x, q.x) + ep) / h);
  const int y0 = (int)floor((fmin(p.y, q.y) - ep) / h), y1 = (int)floor((fmax(p.y, q.y) + ep) / h);
  const int z0 = (int)floor((fmin(p.z, q.z) - ep) / h), z1 = (int)floor((fmax(p.z, q.z) + ep) / h);
  const int mask = c.eeHashSize - 1;
  for (int ix = x0; ix <= x1 && ix <= x0 + 1; ix++)
    for (int iy = y0; iy <= y1 && iy <= y0 + 1; iy++)
      for (int iz = z0; iz <= z1 && iz <= z0 + 1; iz++) {
        const unsigned bk = hash_cell(s, ix, iy, iz, mask);
        if (!FILL) {
          atomicAdd(&c.eeBucketCount[bk], 1);
        } else {
          const int pp = c.eeBucketCount[bk] + atomicAdd(&c.eeBucketCursor[bk], 1);
          c.eeEntry[pp] = x;
        }
      }
}

// One thread per surface edge x: the closest non-adjacent edge y >= x of the
// scene whose closest points lie inside both edges (parameters within
// [1e-4, 1 - 1e-4]; equal distances go to the later edge, as the reference's
// ascending scan keeps the last), kept when no endpoint pair is a surface
// edge and the distance is below eps.  Candidates come from the cells x's own
// box overlaps: any edge within eps of x has a point of its inflated box in
// one of them; farther edges cannot be kept, so the pairs are those of a scan
// over all edges.
__global__ void k_ee_detect(DeviceBatch b, DeviceCollisions c) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= c.nedge) return;
  c.eeSel[x] = -1;
  c.eeKeep[x] = 0;
  c.eeCount[x] = 0;
  const int s = c.edgeScene[x];
  const CollisionScene& cs = c.scenes[s];
  if (!cs.eeOn) return;
  const int2 o = c.edge[x];
  const D3 v0 = pos(b, o.x), v1 = pos(b, o.y);
  const double len0 = norm(v1 - v0);
  int best = -1;
  double bestD = (double)3.402823466e+38f, ab[4] = {-1, -1, -1, -1};
  const double h = ee_cell_size(c, s);
  const D3 bmin = {fmin(v0.x, v1.x), fmin(v0.y, v1.y), fmin(v0.z, v1.z)};
  const D3 bmax = {fmax(v0.x, v1.x), fmax(v0.y, v1.y), fmax(v0.z, v1.z)};
  const int cx0 = (int)floor(fmin(v0.x, v1.x) / h), cx1 = (int)floor(fmax(v0.x, v1.x) / h);
  const int cy0 = (int)floor(fmin(v0.y, v1.y) / h), cy1 = (int)floor(fmax(v0.y, v1.y) / h);
  const int cz0 = (int)floor(fmin(v0.z, v1.z) / h), cz1 = (int)floor(fmax(v0.z, v1.z) / h);
  const int mask = c.eeHashSize - 1;
  for (int ix = cx0; ix <= cx1 && ix <= cx0 + 1; ix++)
  for (int iy = cy0; iy <= cy1 && iy <= cy0 + 1; iy++)
  for (int iz = cz0; iz <= cz1 && iz <= cz0 + 1; iz++) {
  const unsigned bk = hash_cell(s, ix, iy, iz, mask);
  for (int k = c.eeBucketCount[bk]; k < c.eeBucketCount[bk + 1]; k++) {
    const int y = c.eeEntry[k];
    if (y < x || c.edgeScene[y] != s) continue;
    const int2 in = c.edge[y];
    if (o.x == in.x || o.x == in.y || o.y == in.x || o.y == in.y) continue;
    const D3 v2 = pos(b, in.x), v3 = pos(b, in.y);
    // boxes farther apart than eps: farther than eps, never kept (skipping
    // such a candidate cannot change which partner a kept pair has)
    if (fmin(v2.x, v3.x) - cs.eps > bmax.x || fmax(v2.x, v3.x) + cs.eps < bmin.x ||
        fmin(v2.y, v3.y) - cs.eps > bmax.y || fmax(v2.y, v3.y) + cs.eps < bmin.y ||
        fmin(v2.z, v3.z) - cs.eps > bmax.z || fmax(v2.z, v3.z) + cs.eps < bmin.z)
      continue;
    D3 po, pi;
    seg::closest(v0, v1, v2, v3, po, pi);
    const double d = norm(pi - po);
    if (d > bestD || (d == bestD && y <= best)) continue;
    const double a1 = norm(po - v0) / len0, a0 = 1.0 - a1;
    const double b1 = norm(pi - v2) / norm(v3 - v2), b0 = 1.0 - b1;
    const double skip = 1e-4;
    if (a0 < skip || a0 > 1.0 - skip || a1 < skip || a1 > 1.0 - skip) continue;
    if (b0 < skip || b0 > 1.0 - skip || b1 < skip || b1 > 1.0 - skip) continue;
    bestD = d;
    best = y;
    ab[0] = a0, ab[1] = a1, ab[2] = b0, ab[3] = b1;
  }
  }
  if (best < 0) return;
  const int2 in = c.edge[best];
  if (surface_edge(c, cs, o.x, in.x) || surface_edge(c, cs, o.x, in.y) || surface_edge(c, cs, o.y, in.x) ||
      surface_edge(c, cs, o.y, in.y))
    return;
  if (!(bestD < cs.eps)) return;
  bool crossing = false;
  const int2 tt = c.edgeTri[best];
  const int tq[2] = {tt.x, tt.y};
  for (int q = 0; q < 2; q++) {
    if (tq[q] < 0) continue;
    const int* tv = c.tri + 3 * (size_t)tq[q];
    const bool hit = face_edge_cross(pos(b, tv[0]), pos(b, tv[1]), pos(b, tv[2]), v0, v1);
    crossing = crossing || hit;
  }
  c.eeSel[x] = best;
  c.eeKeep[x] = 1;
  c.eeCount[x] = 1;
  c.eeCross[x] = crossing ? 1 : 0;
  c.eeAB[x] = make_double4(ab[0], ab[1], ab[2], ab[3]);
}

// The kept edge pairs after the vertex-face pairs, in edge order:
// EDGE_SQRT_COLLISION with c = (-a0, -a1, b0, b1), diff = sum c_a x_a,
// r = |diff|, n = diff / r, spring = r - eps (r + eps when crossing),
// force -w 2 mu spring c (x) n, clamped Hessian -w (c c^T) (x)
// 2 mu (n n^T + max(spring / r, 0) (I - n n^T)) (the 12x12 eigenvalue clamp
// of (c c^T) (x) G3 clamps G3 alone), zero when r < 1e-7.
__global__ void k_ee_pairs(DeviceBatch b, DeviceCollisions c) {
  const int x = blockIdx.x * blockDim.x + threadIdx.x;
  if (x >= c.nedge || !c.eeKeep[x]) return;
  const int pidx = *c.npairs + c.eeCount[x];
  if (pidx >= c.pairCap) {
    atomicExch(c.overflow, 1);
    return;
  }
  const int s = c.edgeScene[x];
  const CollisionScene& cs = c.scenes[s];
  const int y = c.eeSel[x];
  const int2 o = c.edge[x], in = c.edge[y];
  const int id[4] = {o.x, o.y, in.x, in.y};
  c.pairTet[pidx] = make_int4(o.x, o.y, in.x, in.y);
  const double4 ab = c.eeAB[x];
  const double cvec[4] = {-ab.x, -ab.y, ab.z, ab.w};
  double* C = c.pairC + 4 * (size_t)pidx;
  double* G = c.pairG + 9 * (size_t)pidx;
  double* R = c.pairRhs + 12 * (size_t)pidx;
  double* Fo = c.pairF + 12 * (size_t)pidx;
  for (int a = 0; a < 4; a++) C[a] = cvec[a];
  D3 diff = {0.0, 0.0, 0.0};
  for (int a = 0; a < 4; a++) diff = diff + cvec[a] * pos(b, id[a]);
  const double r = norm(diff);
  if (r < 1e-7) {  // EDGE_SQRT_COLLISION.cpp:_tooSmall
    for (int k = 0; k < 9; k++) G[k] = 0.0;
    for (int k = 0; k < 12; k++) R[k] = Fo[k] = 0.0;
    return;
  }
  const double w = c.edgeArea[x] + c.edgeArea[y];
  const D3 n = (1.0 / r) * diff;
  const double spring = c.eeCross[x] ? r + cs.eps : r - cs.eps;
  const double k2 = fmax(spring / r, 0.0);
  const double n3[3] = {n.x, n.y, n.z};
  const double gs = -w * 2.0 * cs.mu;
  for (int i = 0; i < 3; i++)
    for (int j = 0; j < 3; j++) G[i + 3 * j] = gs * ((1.0 - k2) * n3[i] * n3[j] + (i == j ? k2 : 0.0));
  double zv[3] = {0, 0, 0};
  for (int q = 0; q < 4; q++)
    for (int k = 0; k < 3; k++) zv[k] += cvec[q] * b.v[3 * id[q] + k];
  double Gz[3];
  for (int i = 0; i < 3; i++) Gz[i] = G[i] * zv[0] + G[i + 3] * zv[1] + G[i + 6] * zv[2];
  const double dt = b.scenes[s].dt;
  const int integ = b.scenes[s].integrator;
  double Gn[3] = {0.0, 0.0, 0.0};
  if (integ == kIntegratorNewmark) newmark_coll_term(b, s, id, cvec, G, c.scenes[s].beta, Gn);
  const double fs = gs * spring;
  for (int a = 0; a < 4; a++)
    for (int k = 0; k < 3; k++) {
      Fo[3 * a + k] = fs * cvec[a] * n3[k];
      R[3 * a + k] = integ == kIntegratorPosition ? Fo[3 * a + k]
                     : integ == kIntegratorNewmark ? Fo[3 * a + k] + cvec[a] * Gn[k]
                                                   : dt * (Fo[3 * a + k] + dt * cvec[a] * Gz[k]);
    }
}

__global__ void k_add_total(const int* src, int* dst) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *dst += *src;
}

}  // namespace

// Clears the detection's counters and tables (one kernel, so the detection
// can sit inside a conditional graph body: NEWMARK's Newton loop).  The
// overflow flag is not cleared here: it is cleared once per hobak_batch_step
// call, so an overflow in any step or Newton iteration is reported.
__global__ void k_coll_reset(DeviceCollisions c) {
  const int n = max(max(c.nv + 1, c.hashSize + 1), max(c.eeHashSize + 1, c.nscenes));
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    if (i < c.nscenes) {
      c.cellBits[i] = 0u;
      if (c.nedge > 0) c.eeCellBits[i] = 0u;
    }
    if (i < c.nv) {
      c.vInverted[i] = 0;
      c.incCursor[i] = 0;
    }
    if (i <= c.nv) c.incCount[i] = 0;
    if (i < c.hashSize) c.bucketCursor[i] = 0;
    if (i <= c.hashSize) c.bucketCount[i] = 0;
    if (c.nedge > 0) {
      if (i < c.eeHashSize) c.eeBucketCursor[i] = 0;
      if (i <= c.eeHashSize) c.eeBucketCount[i] = 0;
    }
  }
}

int collision_launches(const DeviceCollisions& c) {
  // reset, inverted, triangles (prepare, 2 bucket passes, scan), vertex
  // query, scan, total, pairs; edges (prepare, 2 bucket passes, scan,
  // detect, scan, pairs, total); incidences (count, scan, fill, sort); the
  // diagonal blocks
  return 1 + 1 + (1 + 2 + 3) + 1 + 3 + 1 + 1 + (c.nedge > 0 ? 1 + 2 + 3 + 1 + 3 + 1 + 1 : 0) + (1 + 3 + 1 + 1) + 1;
}

void launch_collisions(const DeviceBatch& b, const DeviceCollisions& c, cudaStream_t s) {
  {
    const int n = std::max(std::max(c.nv + 1, c.hashSize + 1), std::max(c.eeHashSize + 1, c.nscenes));
    k_coll_reset<<<std::min((n + 255) / 256, 152 * 8), 256, 0, s>>>(c);
  }
  k_mark_inverted<<<(b.nt + 255) / 256, 256, 0, s>>>(b, c);
  k_tri_prepare<<<(c.ntri + 255) / 256, 256, 0, s>>>(b, c);
  k_tri_bucket<false><<<(c.ntri + 255) / 256, 256, 0, s>>>(b, c);
  scan_counts(c.bucketCount, c.hashSize, c.scanTmp, s);
  k_tri_bucket<true><<<(c.ntri + 255) / 256, 256, 0, s>>>(b, c);
  k_vf_query<<<(c.nsv + 127) / 128, 128, 0, s>>>(b, c);
  scan_counts(c.svCount, c.nsv, c.scanTmp, s);
  k_copy_total<<<1, 32, 0, s>>>(c.svCount + c.nsv, c.npairs);
  k_vf_pairs<<<(c.nsv + 127) / 128, 128, 0, s>>>(b, c);
  if (c.nedge > 0) {  // edge-edge pairs follow the vertex-face ones (TIMESTEPPER.cpp:665-690)
    k_edge_prepare<<<(c.nedge + 255) / 256, 256, 0, s>>>(b, c);
    k_edge_bucket<false><<<(c.nedge + 255) / 256, 256, 0, s>>>(b, c);
    scan_counts(c.eeBucketCount, c.eeHashSize, c.scanTmp, s);
    k_edge_bucket<true><<<(c.nedge + 255) / 256, 256, 0, s>>>(b, c);
    k_ee_detect<<<(c.nedge + 127) / 128, 128, 0, s>>>(b, c);
    scan_counts(c.eeCount, c.nedge, c.scanTmp, s);
    k_ee_pairs<<<(c.nedge + 127) / 128, 128, 0, s>>>(b, c);
    k_add_total<<<1, 32, 0, s>>>(c.eeCount + c.nedge, c.npairs);
  }
  k_inc_count<<<(4 * c.pairCap + 255) / 256, 256, 0, s>>>(c);
  scan_counts(c.incCount, c.nv, c.scanTmp, s);
  k_inc_fill<<<(4 * c.pairCap + 255) / 256, 256, 0, s>>>(c);
  k_inc_sort<<<(c.nv + 255) / 256, 256, 0, s>>>(c);
}

void launch_collision_diag(const DeviceBatch& b, const DeviceCollisions& c, cudaStream_t s) {
  k_coll_diag<<<(c.nv + 255) / 256, 256, 0, s>>>(b, c);
}

}  // namespace hobak
