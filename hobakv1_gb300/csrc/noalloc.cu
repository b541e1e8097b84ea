// hobak_element_eval_noalloc: the element-level entry point for callers that
// must not allocate device memory.
//
// Some hosts cannot let a library call cudaMalloc: a plugin inside an
// application that owns the whole device-memory budget (DCC tools, game
// engines, a framework with its own caching pool), or a per-frame loop where
// cudaMalloc/cudaFree would synchronise the device and stall the frame.  This
// variant of hobak_element_eval takes DEVICE pointers for every input and
// output, allocates nothing, and keeps its only scratch -- the per-tet rest
// shape (DmInv, 9 doubles, and rest volume, 1 double) -- in the file-scope
// device array below, which every GPU that loads the library holds until the
// process exits.
//
// Limits and contract:
//   * at most HOBAK_NOALLOC_MAX_TETS tets per call (10 doubles per tet of
//     scratch: 10 MiB); larger calls are rejected with HOBAK_ERR_INVALID;
//   * the first call on a device resolves the array's device address with
//     cudaGetSymbolAddress (once per device, with that device current); make
//     that first call before any stream capture on the device;
//   * every call shares the one array and its contents persist between calls:
//     the rest shape is recomputed on every call and the error word is cleared
//     at the start of every call; calls whose work overlaps on the GPU (other
//     streams, other host threads) race on the array and must be serialised
//     by the caller;
//   * the call returns after its work on `stream` has finished.
#include <cuda_runtime.h>

#include <cstdint>
#include <mutex>
#include <string>

#include "../../include/hobak_gpu.h"
#include "element_math.cuh"
#include "kernels.cuh"

namespace hobak {
// shared with the other entry points so hobak_last_error() reports this call too
int record_error(int code, const std::string& msg);
}  // namespace hobak

namespace {

constexpr int kMaxTets = HOBAK_NOALLOC_MAX_TETS;
constexpr int kMaxDevices = 64;

// [0, 9*kMaxTets): DmInv per tet; [9*kMaxTets, 10*kMaxTets): rest volume;
// then one double holding the error word (first bad tet + 1, or 0).
static __device__ __align__(256) double g_restShapeScratch[10 * kMaxTets + 32];

std::mutex g_setupMutex;
double* g_scratchAddr[kMaxDevices] = {};

// Rest shape of each tet into the scratch array, with the bounds check the
// host-side entry point does on the CPU: a tet naming a vertex outside
// [0, nv) records itself in the error word and is skipped.
__global__ void k_rest_shape_checked(int nv, int nt, const int* __restrict__ tets, const double* __restrict__ rest,
                                     double* scratch) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= nt) return;
  int v[4];
  for (int a = 0; a < 4; a++) {
    v[a] = tets[4 * (size_t)t + a];
    if (v[a] < 0 || v[a] >= nv) {
      unsigned long long* err = reinterpret_cast<unsigned long long*>(scratch + 10 * (size_t)kMaxTets);
      atomicCAS(err, 0ull, (unsigned long long)t + 1ull);
      return;
    }
  }
  double Dm[9];
  for (int a = 0; a < 3; a++)
    for (int i = 0; i < 3; i++) Dm[i + 3 * a] = rest[3 * v[a + 1] + i] - rest[3 * v[0] + i];
  const double c0 = Dm[4] * Dm[8] - Dm[5] * Dm[7];
  const double c1 = Dm[2] * Dm[7] - Dm[1] * Dm[8];
  const double c2 = Dm[1] * Dm[5] - Dm[2] * Dm[4];
  const double det = Dm[0] * c0 + Dm[3] * c1 + Dm[6] * c2;
  const double id = 1.0 / det;
  double* Di = scratch + 9 * (size_t)t;
  Di[0] = c0 * id;
  Di[1] = c1 * id;
  Di[2] = c2 * id;
  Di[3] = (Dm[5] * Dm[6] - Dm[3] * Dm[8]) * id;
  Di[4] = (Dm[0] * Dm[8] - Dm[2] * Dm[6]) * id;
  Di[5] = (Dm[2] * Dm[3] - Dm[0] * Dm[5]) * id;
  Di[6] = (Dm[3] * Dm[7] - Dm[4] * Dm[6]) * id;
  Di[7] = (Dm[1] * Dm[6] - Dm[0] * Dm[7]) * id;
  Di[8] = (Dm[0] * Dm[4] - Dm[1] * Dm[3]) * id;
  scratch[9 * (size_t)kMaxTets + t] = det / 6.0;  // rest volume (TET_MESH.cpp:145-151)
}

int fail(int code, const std::string& msg) { return hobak::record_error(code, msg); }

// Device address of the scratch array for the current device, resolved once.
int scratch_for_current_device(double** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return fail(HOBAK_ERR_NO_DEVICE, std::string("cudaGetDevice: ") + cudaGetErrorString(e));
  if (dev < 0 || dev >= kMaxDevices) return fail(HOBAK_ERR_INVALID, "device ordinal out of range");
  std::lock_guard<std::mutex> lock(g_setupMutex);
  if (!g_scratchAddr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_restShapeScratch);
    if (e != cudaSuccess || !p)
      return fail(HOBAK_ERR_CUDA, std::string("cudaGetSymbolAddress(scratch): ") + cudaGetErrorString(e));
    g_scratchAddr[dev] = static_cast<double*>(p);
  }
  *out = g_scratchAddr[dev];
  return HOBAK_OK;
}

}  // namespace

extern "C" int hobak_element_eval_noalloc(int nv, int nt, const double* rest, const int* tets, const double* x,
                                          const hobak_material* m, double* F, double* sigma, double* force,
                                          double* hessian, void* stream) {
  if (nv <= 0 || nt <= 0 || !rest || !tets || !x || !m) return fail(HOBAK_ERR_INVALID, "bad arguments");
  if (nt > kMaxTets)
    return fail(HOBAK_ERR_INVALID, "hobak_element_eval_noalloc: " + std::to_string(nt) + " tets exceed the " +
                                       std::to_string(kMaxTets) + "-tet scratch limit (HOBAK_NOALLOC_MAX_TETS)");
  if (m->kind < HOBAK_MATERIAL_SNH || m->kind > HOBAK_MATERIAL_ANISOTROPIC_DIRICHLET)
    return fail(HOBAK_ERR_INVALID, "unknown material");
  if (hobak::is_anisotropic(m->kind) &&
      !(m->fiber[0] * m->fiber[0] + m->fiber[1] * m->fiber[1] + m->fiber[2] * m->fiber[2] > 0.0))
    return fail(HOBAK_ERR_INVALID, "anisotropic material needs a non-zero fibre direction");
  if (reinterpret_cast<uintptr_t>(tets) % 16 != 0) return fail(HOBAK_ERR_INVALID, "tets must be 16-byte aligned");
  double* scratch = nullptr;
  int rc = scratch_for_current_device(&scratch);
  if (rc) return rc;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  double* errWord = scratch + 10 * (size_t)kMaxTets;
  cudaError_t e = cudaMemsetAsync(errWord, 0, sizeof(double), s);
  if (e != cudaSuccess) return fail(HOBAK_ERR_CUDA, std::string("clear error word: ") + cudaGetErrorString(e));
  k_rest_shape_checked<<<(nt + 127) / 128, 128, 0, s>>>(nv, nt, tets, rest, scratch);
  unsigned long long bad = 0;
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, errWord, sizeof(bad), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(HOBAK_ERR_CUDA, std::string("rest shape: ") + cudaGetErrorString(e));
  if (bad) return fail(HOBAK_ERR_INVALID, "tet " + std::to_string(bad - 1) + " has a vertex id outside [0, nv)");
  hobak::launch_element_eval(nt, reinterpret_cast<const int4*>(tets), rest, x, scratch, scratch + 9 * (size_t)kMaxTets,
                             m->kind, m->mu, m->lambda, m->fiber, F, sigma, force, hessian, s);
  e = cudaGetLastError();
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (e != cudaSuccess) return fail(HOBAK_ERR_CUDA, std::string("element kernel: ") + cudaGetErrorString(e));
  return HOBAK_OK;
}
