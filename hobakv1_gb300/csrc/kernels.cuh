// Kernel argument blocks and launch wrappers shared by kernels.cu and api.cu.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace hobak {

// Device pointers of one packed batch.  Plain struct passed by value.
struct DeviceBatch {
  int nscenes, nv, nt, nblocks, ntiles;
  const SceneParams* scenes;
  SolveState* solve;
  int* active;  // scenes whose PCG is still running

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

  // tiles
  const int* tileScene;
  const int* tileV0;
  const int* tileV1;

  // per-tet element outputs
  double* elemH;  // [T][90]
  double* elemG;  // [T][12]

  // system and PCG vectors (FP64 path)
  double* lhs;    // [B][9] row major
  double* minv;   // [V][9] row major
  double* rhs;
  double* y;
  double* r;
  double* z;
  double* p0;
  double* p1;
  double* Ap;
  double* partial;  // [ntiles][2]
  double* psi;      // [T] energy density scratch
};

void launch_begin_step(const DeviceBatch& b, cudaStream_t s);
// rawForces = 1 stores the element force f itself in elemG instead of dt (f + dt He v)
void launch_element(const DeviceBatch& b, cudaStream_t s, int rawForces = 0);
// K blocks (column major, un-masked, no mass) and R = sum of element forces, for inspection
void launch_assemble_raw(const DeviceBatch& b, double* K, double* R, cudaStream_t s);
void launch_assemble(const DeviceBatch& b, cudaStream_t s);
void launch_diag_inverse(const DeviceBatch& b, int precond, cudaStream_t s);
void launch_pcg_init(const DeviceBatch& b, cudaStream_t s);
void launch_pcg_iteration(const DeviceBatch& b, const double* pOld, double* pNew, cudaStream_t s);
void launch_spmv(const DeviceBatch& b, const double* pOld, double* pNew, cudaStream_t s);
void launch_update(const DeviceBatch& b, const double* p, cudaStream_t s);
void launch_finish_step(const DeviceBatch& b, cudaStream_t s);
void launch_energy(const DeviceBatch& b, cudaStream_t s);

// element-level entry points (standalone, no batch)
void launch_material_eval(int kind, double mu, double lambda, int n, const double* F, double* psi, double* P,
                          double* H, cudaStream_t s);
void launch_element_eval(int nt, const int4* tets, const double* rest, const double* x, const double* DmInv,
                         const double* vol, int kind, double mu, double lambda, double* F, double* sigma,
                         double* force, double* hessian, cudaStream_t s);

}  // namespace hobak
