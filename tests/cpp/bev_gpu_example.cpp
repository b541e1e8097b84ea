// Drives the C++ mirror (hobakv1_gb300/cpp/HOBAK_GPU.h) the way a reference
// scene drives BACKWARD_EULER_VELOCITY (SIMULATION_SCENE::stepSimulation,
// Scenes/SIMULATION_SCENE.h:120-126): zero external forces, add gravity,
// solve, read position().  Reads a mesh and state from raw binary files and
// writes the final displacement, so a test can compare it with the oracle.
//
//   bev_gpu_example <in.bin> <out.bin> <steps> [position|newmark|stretch]
// ("position" / "newmark" drive BACKWARD_EULER_POSITION / NEWMARK the same way;
// "stretch" runs NEWMARK_STRETCH.h's script: NEWMARK, the surface vertices
// inside two unit cubes pinned to them, the first cube moved 0.01 along -z on
// frames 2..24, no gravity; pinned[] is unused there)
// in.bin: int nv, int nt, int npinned, int material, double mu, lambda,
//         density, dt, rest[3nv], tets[4nt] (int), pinned[npinned] (int), x0[3nv]
#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "../../hobakv1_gb300/cpp/HOBAK_GPU.h"

using namespace HOBAK_GPU;

template <class STEPPER>
int run(TET_MESH& mesh, VOLUME::HYPERELASTIC& material, const double* prm, const std::vector<double>& x0,
        const std::vector<int>& pinned, int steps, const char* out) {
  STEPPER solver(mesh, material);
  solver.setDt(prm[3]);
  solver.scaleMass(prm[2]);
  solver.position() = x0;
  solver.attachKinematicConstraints(pinned);
  const VECTOR3 gravity = {0.0, -9.8 * prm[2], 0.0};
  for (int s = 0; s < steps; s++) {
    std::fill(solver.externalForces().begin(), solver.externalForces().end(), 0.0);
    solver.addGravity(gravity);
    if (!solver.solve(false)) {
      std::fprintf(stderr, "solve failed: %s\n", solver.lastError().c_str());
      return 1;
    }
  }
  FILE* o = std::fopen(out, "wb");
  std::fwrite(solver.position().data(), 8, solver.position().size(), o);
  std::fwrite(solver.velocity().data(), 8, solver.velocity().size(), o);
  std::fclose(o);
  std::printf("%s: steps %d last PCG iterations %d\n", solver.name().c_str(), solver.currentTimestep(),
              solver.lastSolveStats().iterations);
  return 0;
}

// A unit cube kinematic shape (CUBE.cpp:27-55 with KINEMATIC_SHAPE.h:55-69,
// identity rotation and uniform scale).
struct CUBE {
  VECTOR3 translation;
  REAL scale;
  VECTOR3 worldVertexToLocal(const VECTOR3& w) const {
    return {(w[0] - translation[0]) / scale, (w[1] - translation[1]) / scale, (w[2] - translation[2]) / scale};
  }
  VECTOR3 localVertexToWorld(const VECTOR3& l) const {
    return {scale * l[0] + translation[0], scale * l[1] + translation[1], scale * l[2] + translation[2]};
  }
  bool inside(const VECTOR3& p) const {
    const VECTOR3 l = worldVertexToLocal(p);
    for (int i = 0; i < 3; i++)
      if (l[i] > 0.5 || l[i] < -0.5) return false;
    return true;
  }
};

int run_stretch(TET_MESH& mesh, VOLUME::HYPERELASTIC& material, const double* prm, int steps, const char* out) {
  TIMESTEPPER::NEWMARK solver(mesh, material);
  solver.setDt(prm[3]);
  CUBE c0{{0.56, 0.48, -0.24}, 1.0}, c1{{0.56, 0.48, 1.23}, 1.0};
  solver.attachKinematicSurfaceConstraints(&c0);
  solver.attachKinematicSurfaceConstraints(&c1);
  for (int frame = 0; frame < steps; frame++) {
    if (frame > 1 && frame < 25) c0.translation[2] -= 0.01;
    std::fill(solver.externalForces().begin(), solver.externalForces().end(), 0.0);
    if (!solver.solve(false)) {
      std::fprintf(stderr, "solve failed: %s\n", solver.lastError().c_str());
      return 1;
    }
  }
  FILE* o = std::fopen(out, "wb");
  std::fwrite(solver.position().data(), 8, solver.position().size(), o);
  std::fwrite(solver.velocity().data(), 8, solver.velocity().size(), o);
  std::fclose(o);
  return 0;
}

int main(int argc, char** argv) {
  if (argc != 4 && argc != 5) {
    std::fprintf(stderr, "usage: %s in.bin out.bin steps [position]\n", argv[0]);
    return 2;
  }
  FILE* f = std::fopen(argv[1], "rb");
  if (!f) return 2;
  int hdr[4];
  double prm[4];
  if (std::fread(hdr, sizeof(int), 4, f) != 4 || std::fread(prm, sizeof(double), 4, f) != 4) return 2;
  const int nv = hdr[0], nt = hdr[1], np = hdr[2], kind = hdr[3];
  std::vector<double> rest(3 * nv), x0(3 * nv);
  std::vector<int> tets(4 * nt), pinned(np);
  if (std::fread(rest.data(), 8, rest.size(), f) != rest.size() || std::fread(tets.data(), 4, tets.size(), f) != tets.size() ||
      std::fread(pinned.data(), 4, pinned.size(), f) != pinned.size() || std::fread(x0.data(), 8, x0.size(), f) != x0.size())
    return 2;
  std::fclose(f);

  std::vector<VECTOR3> restV(nv);
  for (int i = 0; i < nv; i++) restV[i] = {rest[3 * i], rest[3 * i + 1], rest[3 * i + 2]};
  std::vector<VECTOR4I> tetV(nt);
  for (int t = 0; t < nt; t++) tetV[t] = {tets[4 * t], tets[4 * t + 1], tets[4 * t + 2], tets[4 * t + 3]};
  TET_MESH mesh(restV, tetV);
  VOLUME::SNH snh(prm[0], prm[1]);
  VOLUME::ARAP arap(prm[0], prm[1]);
  VOLUME::HYPERELASTIC& material = (kind == HOBAK_MATERIAL_ARAP) ? (VOLUME::HYPERELASTIC&)arap : snh;

  const int steps = std::atoi(argv[3]);
  if (argc == 5 && std::string(argv[4]) == "stretch") return run_stretch(mesh, material, prm, steps, argv[2]);
  if (argc == 5 && std::string(argv[4]) == "position")
    return run<TIMESTEPPER::BACKWARD_EULER_POSITION>(mesh, material, prm, x0, pinned, steps, argv[2]);
  if (argc == 5 && std::string(argv[4]) == "newmark")
    return run<TIMESTEPPER::NEWMARK>(mesh, material, prm, x0, pinned, steps, argv[2]);
  return run<TIMESTEPPER::BACKWARD_EULER_VELOCITY>(mesh, material, prm, x0, pinned, steps, argv[2]);
}
