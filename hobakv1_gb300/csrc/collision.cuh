// Vertex-face self-collision data of a batch (device side).
//
// Surfaces are extracted once on the host (TET_MESH.cpp:294-350 order and
// winding); every step the GPU rebuilds a spatial hash of the surface
// triangles, runs the reference's narrow phase per surface vertex, and turns
// each (vertex, triangle) pair into a collision tet with a spring force and an
// eigen-clamped Hessian (VERTEX_FACE_SQRT_COLLISION).  All lists are built in
// a fixed order (pairs sorted by scene, surface vertex, triangle; per-vertex
// incidences sorted by pair), so results are deterministic.
#pragma once
#include <cuda_runtime.h>

namespace hobak {

constexpr int kMaxPairsPerVertex = 16;  // candidate triangles kept per surface vertex

struct CollisionScene {
  int vfOn;
  int tri0, ntri;   // surface triangle range
  int sv0, nsv;     // surface vertex range
  double eps, mu, beta;
  int eeOn;         // edge-edge self collisions (same eps, mu, beta)
  int e0, ne;       // surface edge range
};

struct DeviceCollisions {
  int nscenes, ntri, nsv, nv, hashSize, pairCap;
  const CollisionScene* scenes;
  // surface (static)
  const int* tri;          // [ntri][3] global vertex ids, reference winding
  const int* triScene;     // [ntri]
  const double* triArea;   // [ntri] rest area
  const int* triNbr;       // [ntri][3] neighbouring triangle across edge (j, j+1)
  const int* sv;           // [nsv] global vertex ids, ascending per scene
  const int* svScene;      // [nsv]
  const double* svArea;    // [nsv] rest one-ring area
  int nedge;
  const int2* edge;        // [nedge] surface edges (lo, hi), global ids, ascending per scene
  const int* edgeScene;    // [nedge]
  const double* edgeArea;  // [nedge] a third of each adjacent triangle's rest area
  const int2* edgeTri;     // [nedge] first two adjacent surface triangles (-1: none)
  // per step
  unsigned* cellBits;      // [nscenes] largest triangle extent (float bits) -> cell size
  unsigned char* vInverted;  // [nv]
  unsigned char* triSkip;    // [ntri] degenerate or all-inverted
  int* bucketCount;        // [hashSize + 1] then exclusive scan
  int* bucketCursor;       // [hashSize]
  int* entryTri;           // [8 * ntri]
  int* svCount;            // [nsv + 1] then exclusive scan
  int* svCand;             // [nsv][kMaxPairsPerVertex]
  int* overflow;           // [1] set when a vertex had more candidates than fit
  int* npairs;             // [1]
  int4* pairTet;           // [pairCap] collision tet (v, f2, f1, f0)
  double* pairC;           // [pairCap][4] (1, -b0, -b1, -b2)
  double* pairG;           // [pairCap][9] 3x3 factor of the clamped Hessian, times -w 2 mu
  double* pairRhs;         // [pairCap][12] dt (f + dt H v)
  double* pairF;           // [pairCap][12] collision force -w grad psi (for inspection)
  double* diag;            // [nv][9] vertex's own 3x3 block of -(dt beta + dt^2) H_coll (FP64)
  int* incCount;           // [nv + 1] then exclusive scan
  int* incCursor;          // [nv]
  int* incList;            // [4 * pairCap] pair * 4 + slot
  int* scanTmp;            // block sums for the device-wide scans
  // edge-edge, per step: each surface edge's closest admissible partner
  int* eeSel;              // [nedge] partner edge or -1
  unsigned char* eeKeep;   // [nedge] 1: the pair is a collision
  unsigned char* eeCross;  // [nedge] 1: the edge crosses a triangle next to its partner
  double4* eeAB;           // [nedge] (a0, a1, b0, b1)
  int* eeCount;            // [nedge + 1] keep flags, then exclusive scan
  // edge-edge broad phase: each edge's eps-inflated box hashed into cells no
  // smaller than the scene's largest inflated edge extent (<= 8 cells each)
  int eeHashSize;
  unsigned* eeCellBits;    // [nscenes] largest inflated edge extent (float bits)
  int* eeBucketCount;      // [eeHashSize + 1] then exclusive scan
  int* eeBucketCursor;     // [eeHashSize]
  int* eeEntry;            // [8 * nedge]
};

struct DeviceBatch;

// Enqueue the per-step detection and response (after the element kernel,
// before assembly uses them).  dtScale: per-scene dt taken from the batch.
void launch_collisions(const DeviceBatch& b, const DeviceCollisions& c, cudaStream_t s);
// The vertices' own collision blocks (DeviceCollisions::diag, FP64), before
// the preconditioner reads them.
void launch_collision_diag(const DeviceBatch& b, const DeviceCollisions& c, cudaStream_t s);
// kernels that launch_collisions and launch_collision_diag enqueue per detection
int collision_launches(const DeviceCollisions& c);

}  // namespace hobak
