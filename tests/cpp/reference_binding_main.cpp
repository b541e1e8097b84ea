// Drives BACKWARD_EULER_VELOCITY_GPU (hobakv1_gb300/cpp/hobak_binding/), the
// binding a HOBAK maintainer adds, the way a reference scene drives a
// TIMESTEPPER (SIMULATION_SCENE::stepSimulation, Scenes/SIMULATION_SCENE.h:
// 120-126): HOBAK's own TET_MESH_FASTER, SNH and CUBE, pins attached through
// attachKinematicConstraints, gravity through addGravity, scaleMass, then
// solve().  Built against the reference's headers and objects plus
// libhobak_gpu.so.  Prints "solve ok <iterations> <|x|>" or
// "solve failed: <the library's message>" and returns 0 either way (a host
// without a GPU reports that it has none).
//
//   reference_binding_main [N] [steps]
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "Geometry/CUBE.h"
#include "Geometry/TET_MESH_FASTER.h"
#include "Hyperelastic/Volume/SNH.h"
#include "hobak_binding/BACKWARD_EULER_VELOCITY_GPU.h"

using namespace HOBAK;

int main(int argc, char** argv) {
  const int N = argc > 1 ? std::atoi(argv[1]) : 4;
  const int steps = argc > 2 ? std::atoi(argv[2]) : 2;
  // Kuhn-split unit cube: six tets per cell around the main diagonal
  std::vector<VECTOR3> rest;
  std::vector<VECTOR4I> tets;
  const int n1 = N + 1;
  for (int k = 0; k < n1; k++)
    for (int j = 0; j < n1; j++)
      for (int i = 0; i < n1; i++) rest.push_back(VECTOR3(i, j, k) / N);
  const int perm[6][3] = {{0, 1, 2}, {1, 2, 0}, {2, 0, 1}, {0, 2, 1}, {2, 1, 0}, {1, 0, 2}};
  const int sign[6] = {1, 1, 1, -1, -1, -1};
  auto id = [&](int i, int j, int k) { return i + n1 * (j + n1 * k); };
  for (int k = 0; k < N; k++)
    for (int j = 0; j < N; j++)
      for (int i = 0; i < N; i++)
        for (int p = 0; p < 6; p++) {
          int c[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {1, 1, 1}};
          c[1][perm[p][0]] = 1;
          c[2][perm[p][0]] = 1;
          c[2][perm[p][1]] = 1;
          int v[4];
          for (int a = 0; a < 4; a++) v[a] = id(i + c[a][0], j + c[a][1], k + c[a][2]);
          if (sign[p] < 0) std::swap(v[1], v[2]);
          tets.push_back(VECTOR4I(v[0], v[1], v[2], v[3]));
        }
  TET_MESH_FASTER mesh(rest, tets);
  const REAL E = 1e3, nu = 0.45;
  const REAL mu = VOLUME::HYPERELASTIC::computeMu(E, nu), lambda = VOLUME::HYPERELASTIC::computeLambda(E, nu);
  VOLUME::SNH snh(mu, lambda);
  hobak_material m{HOBAK_MATERIAL_SNH, mu, lambda, {0.0, 0.0, 0.0}};
  TIMESTEPPER::BACKWARD_EULER_VELOCITY_GPU solver(mesh, snh, m);
  solver.vertexFaceSelfCollisionsOn() = false;
  solver.edgeEdgeSelfCollisionsOn() = false;
  const REAL density = 1000.0;
  solver.scaleMass(density);
  // pin the top layer (y = 1) with a cube that holds only it
  CUBE top(VECTOR3(0.5, 1.0, 0.5), 0.5 / N);
  solver.attachKinematicConstraints(&top);
  for (int s = 0; s < steps; s++) {
    solver.externalForces().setZero();
    solver.addGravity(VECTOR3(0.0, -9.8 * density, 0.0));
    if (!solver.solve(false)) {
      std::printf("solve failed: %s\n", solver.lastError());
      return 0;
    }
  }
  std::printf("solve ok %d %.17g\n", (int)solver.constrainedNodes().size(), solver.position().norm());
  return 0;
}
