// BACKWARD_EULER_VELOCITY_GPU: the timestepper a HOBAK maintainer adds to
// HOBAK (as Timestepper/BACKWARD_EULER_VELOCITY_GPU.h) to run
// BACKWARD_EULER_VELOCITY::solve (BACKWARD_EULER_VELOCITY.cpp:107-235) on a
// GB300 through the C ABI of include/hobak_gpu.h.  It derives from HOBAK's own
// TIMESTEPPER (Timestepper/TIMESTEPPER.h:37-219), so scenes, recorders and
// callers keep using position(), velocity(), externalForces(), the collision
// switches, addGravity(), attachKinematicConstraints() and scaleMass()
// unchanged; HOBAK's host state stays the source of truth and is uploaded
// before and downloaded after every step.  Link with libhobak_gpu.so.
#ifndef BACKWARD_EULER_VELOCITY_GPU_H
#define BACKWARD_EULER_VELOCITY_GPU_H

#include <cstdio>
#include <vector>

#include "Timestepper/TIMESTEPPER.h"
#include "hobak_gpu.h"

namespace HOBAK {
namespace TIMESTEPPER {

class BACKWARD_EULER_VELOCITY_GPU : public TIMESTEPPER {
 public:
  // HOBAK's materials keep (mu, lambda) private (SNH.h:47-49), so the caller
  // also passes the descriptor it constructed the material with, e.g.
  // hobak_material{HOBAK_MATERIAL_SNH, mu, lambda, {0, 0, 0}} for SNH(mu, lambda).
  BACKWARD_EULER_VELOCITY_GPU(TET_MESH& tetMesh, VOLUME::HYPERELASTIC& hyperelastic, const hobak_material& material,
                              const hobak_solver_opts* opts = nullptr)
      : TIMESTEPPER(tetMesh, hyperelastic), _material(material) {
    _dt = 1.0 / 60.0;  // BACKWARD_EULER_VELOCITY.cpp:37
    _name = std::string("BACKWARD_EULER_VELOCITY_GPU");
    hobak_default_solver_opts(&_opts);
    if (opts) _opts = *opts;
  }
  ~BACKWARD_EULER_VELOCITY_GPU() override {
    if (_handle) hobak_gpu_destroy(_handle);
  }

  bool solve(const bool verbose) override {
    _positionOld = _position;  // BACKWARD_EULER_VELOCITY.cpp:122
    if (!_handle && !build()) return false;
    if (!pushCollisionSwitches()) return false;
    // moving kinematic shapes: pin targets from the shapes, as
    // applyKinematicConstraints does at every solve (TIMESTEPPER.cpp:105-122)
    if (!_kinematicConstraints.empty()) {
      const std::vector<VECTOR3>& rest = _tetMesh.restVertices();
      for (size_t k = 0; k < _kinematicConstraints.size(); k++) {
        const KINEMATIC_CONSTRAINT& c = _kinematicConstraints[k];
        const VECTOR3 d = c.shape->localVertexToWorld(c.localPosition) - rest[c.vertexID];
        for (int i = 0; i < 3; i++) _targets[3 * k + i] = d[i];
      }
      if (hobak_batch_set_pin_targets(_handle, 0, _targets.data()) != HOBAK_OK) return false;
    }
    if (hobak_gpu_set_state(_handle, _position.data(), _velocity.data()) != HOBAK_OK ||
        hobak_gpu_set_external_forces(_handle, _externalForces.data()) != HOBAK_OK)
      return false;
    hobak_step_stats st;
    if (hobak_gpu_step(_handle, 1, &st) < 0) return false;
    if (hobak_gpu_get_state(_handle, _position.data(), _velocity.data()) != HOBAK_OK) return false;
    _tetMesh.setDisplacement(_position);  // BACKWARD_EULER_VELOCITY.cpp:227
    _seenPCGIterations = st.iterations;
    _residual = st.rel_residual;
    if (verbose) std::printf("  PCG iters: %3i err: %6.4e \n", st.iterations, st.rel_residual);
    return true;
  }

  // why the last solve() returned false (the library's message)
  const char* lastError() const { return hobak_last_error(); }

 protected:
  // the device applies the pin targets itself (set in solve())
  void updateConstraintTargets() override {}

 private:
  bool build() {
    const std::vector<VECTOR3>& restV = _tetMesh.restVertices();
    std::vector<double> rest;
    std::vector<int> tets, pins;
    rest.reserve(3 * restV.size());
    for (const VECTOR3& v : restV) rest.insert(rest.end(), {v[0], v[1], v[2]});
    for (const VECTOR4I& t : _tetMesh.tets()) tets.insert(tets.end(), {t[0], t[1], t[2], t[3]});
    for (const KINEMATIC_CONSTRAINT& c : _kinematicConstraints) pins.push_back(c.vertexID);
    _targets.assign(3 * pins.size(), 0.0);
    // _M = diag(one-ring volume), scaled by scaleMass() (TIMESTEPPER.cpp:176-208,
    // TIMESTEPPER.h:100): the scale from the sums of both, so no single vertex
    // (which may have a zero one-ring volume) decides it
    double oneRing = 0.0;
    for (const REAL r : _tetMesh.restOneRingVolumes()) oneRing += r;
    const double density = _M.diagonal().sum() / (3.0 * oneRing);
    hobak_scene_desc d{};
    d.nv = (int)restV.size();
    d.nt = (int)_tetMesh.tets().size();
    d.rest = rest.data();
    d.tets = tets.data();
    d.material = _material;
    d.density = density;  // gravity arrives through externalForces() (addGravity)
    d.dt = _dt;
    d.npinned = (int)pins.size();
    d.pinned = pins.empty() ? nullptr : pins.data();
    d.x0 = _position.data();
    d.v0 = _velocity.data();
    return hobak_gpu_create(&d, &_opts, &_handle) == HOBAK_OK;
  }

  // HOBAK's collision switches are public references that scenes set after
  // construction; both are on by default (TIMESTEPPER.cpp:83-84)
  bool pushCollisionSwitches() {
    const int vf = _vertexFaceSelfCollisionsOn ? 1 : 0, ee = _edgeEdgeSelfCollisionsOn ? 1 : 0;
    const double eps = _tetMesh.collisionEps();
    if (vf == 0 && ee == 0 && _vf <= 0 && _ee <= 0) {  // off, and never turned on: nothing to build
      _vf = _ee = 0;
      return true;
    }
    if (vf == _vf && ee == _ee && eps == _eps && _collisionStiffness == _mu && _collisionDampingBeta == _beta)
      return true;
    if (hobak_gpu_set_collisions(_handle, vf, eps, _collisionStiffness, _collisionDampingBeta) != HOBAK_OK ||
        hobak_gpu_set_edge_collisions(_handle, ee) != HOBAK_OK)
      return false;
    _vf = vf;
    _ee = ee;
    _eps = eps;
    _mu = _collisionStiffness;
    _beta = _collisionDampingBeta;
    return true;
  }

  hobak_material _material;
  hobak_solver_opts _opts;
  hobak_batch _handle = nullptr;
  std::vector<double> _targets;
  int _vf = -1, _ee = -1;
  double _eps = -1.0, _mu = -1.0, _beta = -1.0;
};

}  // namespace TIMESTEPPER
}  // namespace HOBAK

#endif
