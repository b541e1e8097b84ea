// C++ host mirror of HOBAK's hot-path interfaces over the GB300 C ABI
// (include/hobak_gpu.h).  Header only; link with libhobak_gpu.so.
//
// Names and argument meaning follow the reference so a caller can switch by
// changing the namespace:
//   HOBAK::VOLUME::HYPERELASTIC and energies  -> HOBAK_GPU::VOLUME::*
//     (Hyperelastic/Volume/HYPERELASTIC.h:31-64; SNH.h, ARAP.h, STVK.h, ...)
//   HOBAK::TET_MESH                           -> HOBAK_GPU::TET_MESH
//   HOBAK::TIMESTEPPER::BACKWARD_EULER_VELOCITY
//                                             -> HOBAK_GPU::TIMESTEPPER::BACKWARD_EULER_VELOCITY
//     (Timestepper/TIMESTEPPER.h:37-219, BACKWARD_EULER_VELOCITY.h:35-58)
// Vectors are std::vector<double> (interleaved xyz) instead of Eigen types;
// 3x3 matrices are 9 doubles in the reference's column-major flatten order.
// Like the reference, nothing throws: solve() returns false on failure and
// lastError() says why.
#pragma once

#include <algorithm>
#include <array>
#include <cmath>
#include <functional>
#include <map>
#include <string>
#include <vector>

#include "../../include/hobak_gpu.h"

namespace HOBAK_GPU {

typedef double REAL;
typedef std::vector<REAL> VECTOR;
typedef std::array<REAL, 3> VECTOR3;
typedef std::array<int, 4> VECTOR4I;

namespace VOLUME {

class HYPERELASTIC {
 public:
  HYPERELASTIC(int kind, REAL mu, REAL lambda) : _material{kind, mu, lambda, {0.0, 0.0, 0.0}} {}
  virtual ~HYPERELASTIC() = default;
  virtual std::string name() const = 0;

  // energyNeedsSVD() / PK1NeedsSVD() (HYPERELASTIC.h:56-59)
  bool energyNeedsSVD() const {
    int e = 0, p = 0;
    hobak_material_needs_svd(_material.kind, &e, &p);
    return e != 0;
  }
  bool PK1NeedsSVD() const {
    int e = 0, p = 0;
    hobak_material_needs_svd(_material.kind, &e, &p);
    return p != 0;
  }
  // hessian(F) (HYPERELASTIC.h:44): unclamped, 81 doubles column major
  bool hessian(const REAL* F, REAL* H) const { return hobak_material_hessian(&_material, 1, F, H) == HOBAK_OK; }
  // The (U, Sigma, V) overloads (HYPERELASTIC.h:37-49); NULL outputs skip
  bool evaluate(const REAL* U, const REAL* Sigma, const REAL* V, REAL* psi, REAL* P, REAL* H,
                REAL* clampedH) const {
    return hobak_material_eval_svd(&_material, 1, U, Sigma, V, psi, P, H, clampedH) == HOBAK_OK;
  }

  // Single-F forms (HYPERELASTIC.h:36-48); F, P column major (flatten order).
  REAL psi(const REAL* F) const {
    REAL out = 0;
    return hobak_material_eval(&_material, 1, F, &out, nullptr, nullptr) == HOBAK_OK ? out : NAN;
  }
  bool PK1(const REAL* F, REAL* P) const { return hobak_material_eval(&_material, 1, F, nullptr, P, nullptr) == 0; }
  bool clampedHessian(const REAL* F, REAL* H) const {
    return hobak_material_eval(&_material, 1, F, nullptr, nullptr, H) == HOBAK_OK;
  }
  // Batched forms: n gradients at once (9n in; n, 9n, 81n out; NULL skips).
  bool evaluate(int n, const REAL* F, REAL* psi, REAL* P, REAL* H) const {
    return hobak_material_eval(&_material, n, F, psi, P, H) == HOBAK_OK;
  }

  // HYPERELASTIC::computeMu / computeLambda (HYPERELASTIC.cpp:111-122)
  static REAL computeMu(const REAL E, const REAL nu) { return E / (2.0 * (1.0 + nu)); }
  static REAL computeLambda(const REAL E, const REAL nu) { return (E * nu) / ((1.0 + nu) * (1.0 - 2.0 * nu)); }

  const hobak_material& descriptor() const { return _material; }

 protected:
  hobak_material _material;
};

class SNH : public HYPERELASTIC {
 public:
  SNH(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_SNH, mu, lambda) {}
  std::string name() const override { return "SNH"; }
};
class ARAP : public HYPERELASTIC {
 public:
  ARAP(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_ARAP, mu, lambda) {}
  std::string name() const override { return "ARAP"; }
};
class STVK : public HYPERELASTIC {
 public:
  STVK(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_STVK, mu, lambda) {}
  std::string name() const override { return "STVK"; }
};
class LINEAR : public HYPERELASTIC {
 public:
  LINEAR(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_LINEAR, mu, lambda) {}
  std::string name() const override { return "LINEAR"; }
};
class NEO_HOOKEAN_BW : public HYPERELASTIC {
 public:
  NEO_HOOKEAN_BW(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_NEO_HOOKEAN_BW, mu, lambda) {}
  std::string name() const override { return "NEO_HOOKEAN_BW"; }
};
class SNH_WITH_BARRIER : public HYPERELASTIC {
 public:
  SNH_WITH_BARRIER(const REAL& mu, const REAL& lambda) : HYPERELASTIC(HOBAK_MATERIAL_SNH_BARRIER, mu, lambda) {}
  std::string name() const override { return "SNH_WITH_BARRIER"; }
};

// The anisotropic energies take (mu, a) like ANISOTROPIC_ARAP(mu, a)
// (ANISOTROPIC_ARAP.h:28); the library normalises a.
class ANISOTROPIC : public HYPERELASTIC {
 public:
  ANISOTROPIC(int kind, const REAL& mu, const VECTOR3& a) : HYPERELASTIC(kind, mu, 0.0) {
    for (int i = 0; i < 3; i++) _material.fiber[i] = a[i];
  }
};
class ANISOTROPIC_ARAP : public ANISOTROPIC {
 public:
  ANISOTROPIC_ARAP(const REAL& mu, const VECTOR3& a) : ANISOTROPIC(HOBAK_MATERIAL_ANISOTROPIC_ARAP, mu, a) {}
  std::string name() const override { return "ANISOTROPIC_ARAP"; }
};
class ANISOTROPIC_STVK : public ANISOTROPIC {
 public:
  ANISOTROPIC_STVK(const REAL& mu, const VECTOR3& a) : ANISOTROPIC(HOBAK_MATERIAL_ANISOTROPIC_STVK, mu, a) {}
  std::string name() const override { return "ANISOTROPIC_STVK"; }
};
class ANISOTROPIC_FUNG : public ANISOTROPIC {
 public:
  ANISOTROPIC_FUNG(const REAL& mu, const VECTOR3& a) : ANISOTROPIC(HOBAK_MATERIAL_ANISOTROPIC_FUNG, mu, a) {}
  std::string name() const override { return "ANISOTROPIC_FUNG"; }
};
class ANISOTROPIC_DIRICHLET : public ANISOTROPIC {
 public:
  ANISOTROPIC_DIRICHLET(const REAL& mu, const VECTOR3& a)
      : ANISOTROPIC(HOBAK_MATERIAL_ANISOTROPIC_DIRICHLET, mu, a) {}
  std::string name() const override { return "ANISOTROPIC_DIRICHLET"; }
};

// VOLUME::GREEN_DAMPING(mu) (Damping/Volume/GREEN_DAMPING.h): the damping
// of NEWMARK's energy-damped solve, P = mu F (F^T Fdot + Fdot^T F)
// (GREEN_DAMPING.cpp:46-50); evaluated on the device inside the step.
class GREEN_DAMPING {
 public:
  explicit GREEN_DAMPING(const REAL& mu) : _mu(mu) {}
  std::string name() const { return "GREEN_DAMPING"; }
  REAL mu() const { return _mu; }

 private:
  REAL _mu;
};

}  // namespace VOLUME

// Rest mesh (TET_MESH.h): rest vertices and tets, plus the displacement the
// timestepper starts from.
class TET_MESH {
 public:
  TET_MESH(const std::vector<VECTOR3>& restVertices, const std::vector<VECTOR4I>& tets)
      : _rest(restVertices), _tets(tets), _displacement(3 * restVertices.size(), 0.0) {
    _oneRing.assign(_rest.size(), 0.0);
    for (const auto& t : _tets) {
      const REAL v = volume(t);
      for (int a = 0; a < 4; a++) _oneRing[t[a]] += 0.25 * v;
    }
  }
  const std::vector<VECTOR3>& restVertices() const { return _rest; }
  const std::vector<VECTOR4I>& tets() const { return _tets; }
  const std::vector<REAL>& restOneRingVolumes() const { return _oneRing; }
  int totalVertices() const { return (int)_rest.size(); }
  int DOFs() const { return 3 * (int)_rest.size(); }
  // vertices of the faces that belong to one tet only, ascending
  // (TET_MESH::computeSurfaceVertices, TET_MESH.cpp:567-590)
  std::vector<int> surfaceVertices() const {
    std::map<std::array<int, 3>, int> faces;
    static const int kFace[4][3] = {{0, 1, 2}, {0, 1, 3}, {0, 2, 3}, {1, 2, 3}};
    for (const auto& t : _tets)
      for (const auto& f : kFace) {
        std::array<int, 3> k = {t[f[0]], t[f[1]], t[f[2]]};
        std::sort(k.begin(), k.end());
        faces[k]++;
      }
    std::vector<int> out;
    for (const auto& kv : faces)
      if (kv.second == 1) out.insert(out.end(), kv.first.begin(), kv.first.end());
    std::sort(out.begin(), out.end());
    out.erase(std::unique(out.begin(), out.end()), out.end());
    return out;
  }
  void setDisplacement(const VECTOR& delta) { _displacement = delta; }
  VECTOR getDisplacement() const { return _displacement; }

 private:
  REAL volume(const VECTOR4I& t) const {
    const VECTOR3 &a = _rest[t[0]], &b = _rest[t[1]], &c = _rest[t[2]], &d = _rest[t[3]];
    const REAL d1[3] = {b[0] - a[0], b[1] - a[1], b[2] - a[2]};
    const REAL d2[3] = {c[0] - a[0], c[1] - a[1], c[2] - a[2]};
    const REAL d3[3] = {d[0] - a[0], d[1] - a[1], d[2] - a[2]};
    return (d3[0] * (d1[1] * d2[2] - d1[2] * d2[1]) + d3[1] * (d1[2] * d2[0] - d1[0] * d2[2]) +
            d3[2] * (d1[0] * d2[1] - d1[1] * d2[0])) / 6.0;
  }
  std::vector<VECTOR3> _rest;
  std::vector<VECTOR4I> _tets;
  std::vector<REAL> _oneRing;
  VECTOR _displacement;
};

namespace TIMESTEPPER {

// GPU drop-in for BACKWARD_EULER_VELOCITY.  position() / velocity() /
// externalForces() are host state that solve() uploads, steps on the GPU and
// downloads, so callers that edit or read them between steps (scenes,
// recorders) see the reference's semantics.  Settings are frozen at the first
// solve().
class BACKWARD_EULER_VELOCITY {
 public:
  BACKWARD_EULER_VELOCITY(TET_MESH& tetMesh, VOLUME::HYPERELASTIC& hyperelastic)
      : _tetMesh(tetMesh), _hyperelastic(hyperelastic) {
    const int n = tetMesh.DOFs();
    _position = tetMesh.getDisplacement();
    _velocity.assign(n, 0.0);
    _externalForces.assign(n, 0.0);
    hobak_default_solver_opts(&_opts);
  }
  ~BACKWARD_EULER_VELOCITY() {
    if (_handle) hobak_gpu_destroy(_handle);
  }
  BACKWARD_EULER_VELOCITY(const BACKWARD_EULER_VELOCITY&) = delete;
  BACKWARD_EULER_VELOCITY& operator=(const BACKWARD_EULER_VELOCITY&) = delete;

  VECTOR& position() { return _position; }
  VECTOR& velocity() { return _velocity; }
  VECTOR& externalForces() { return _externalForces; }
  const std::string& name() const { return _name; }
  REAL dt() const { return _dt; }
  void setDt(const REAL dt) { _dt = dt; }
  void scaleMass(const REAL& scalar) { _massScale *= scalar; }
  void setSolverOptions(const hobak_solver_opts& o) { _opts = o; }

  // f_ext += oneRingVolume * bodyForce (TIMESTEPPER.cpp:334-345)
  void addGravity(const VECTOR3& bodyForce) {
    const auto& v = _tetMesh.restOneRingVolumes();
    for (size_t x = 0; x < v.size(); x++)
      for (int i = 0; i < 3; i++) _externalForces[3 * x + i] += v[x] * bodyForce[i];
  }
  // Pin vertices at their current positions (TIMESTEPPER.cpp:380-403); any
  // shape type with bool inside(const VECTOR3&) works, as does a list of ids.
  // A shape that also has VECTOR3 worldVertexToLocal(const VECTOR3&) and
  // localVertexToWorld(const VECTOR3&) (KINEMATIC_SHAPE.h:55-69) carries its
  // pins along when it moves between solves.
  template <typename SHAPE>
  void attachKinematicConstraints(const SHAPE* shape) {
    std::vector<int> all(_tetMesh.totalVertices());
    for (size_t x = 0; x < all.size(); x++) all[x] = (int)x;
    attachShape(shape, all, 0);
  }
  // The surface vertices inside the shape (TIMESTEPPER.cpp:350-375).
  template <typename SHAPE>
  void attachKinematicSurfaceConstraints(const SHAPE* shape) {
    attachShape(shape, _tetMesh.surfaceVertices(), 0);
  }
  void attachKinematicConstraints(const std::vector<int>& vertexIDs) {
    _pinned.insert(_pinned.end(), vertexIDs.begin(), vertexIDs.end());
  }

  // One BACKWARD_EULER_VELOCITY::solve step (BACKWARD_EULER_VELOCITY.cpp:96-235) on the GPU.
  bool solve(const bool verbose) {
    if (!_handle && !build()) return false;
    if (hobak_gpu_set_state(_handle, _position.data(), _velocity.data()) != HOBAK_OK ||
        hobak_batch_set_external_forces(_handle, 0, _externalForces.data()) != HOBAK_OK || !pushPinTargets())
      return fail();
    const int rc = hobak_gpu_step(_handle, 1, &_stats);
    if (rc < 0) return fail();
    if (hobak_gpu_get_state(_handle, _position.data(), _velocity.data()) != HOBAK_OK) return fail();
    _currentTimestep++;
    _time += _dt;
    if (verbose) std::printf("  PCG iters: %3i err: %6.4e \n", _stats.iterations, _stats.rel_residual);
    return true;
  }

  const hobak_step_stats& lastSolveStats() const { return _stats; }
  const std::string& lastError() const { return _error; }
  int currentTimestep() const { return _currentTimestep; }

 protected:
  template <typename SHAPE>
  auto attachShape(const SHAPE* shape, const std::vector<int>& candidates, int)
      -> decltype(shape->worldVertexToLocal(VECTOR3{}), shape->localVertexToWorld(VECTOR3{}), void()) {
    const auto& rest = _tetMesh.restVertices();
    for (int x : candidates) {
      const VECTOR3 p = {rest[x][0] + _position[3 * x], rest[x][1] + _position[3 * x + 1],
                         rest[x][2] + _position[3 * x + 2]};
      if (!shape->inside(p)) continue;
      _pinned.push_back(x);
      const VECTOR3 local = shape->worldVertexToLocal(p);
      // later constraints on a vertex override earlier ones (TIMESTEPPER.cpp:105-122)
      _shapePins[x] = [shape, local]() { return shape->localVertexToWorld(local); };
    }
  }
  template <typename SHAPE>
  void attachShape(const SHAPE* shape, const std::vector<int>& candidates, long) {
    const auto& rest = _tetMesh.restVertices();
    for (int x : candidates) {
      const VECTOR3 p = {rest[x][0] + _position[3 * x], rest[x][1] + _position[3 * x + 1],
                         rest[x][2] + _position[3 * x + 2]};
      if (shape->inside(p)) _pinned.push_back(x);
    }
  }
  // applyKinematicConstraints (TIMESTEPPER.cpp:105-122): each shape-held
  // pin's target displacement from the shape's current transform
  bool pushPinTargets() {
    if (_shapePins.empty()) return true;
    const auto& rest = _tetMesh.restVertices();
    std::vector<REAL> t(3 * _pinned.size());
    for (size_t k = 0; k < _pinned.size(); k++) {
      const int u = _pinned[k];
      auto it = _shapePins.find(u);
      for (int i = 0; i < 3; i++)
        t[3 * k + i] = it != _shapePins.end() ? it->second()[i] - rest[u][i] : _pinnedAt[3 * k + i];
    }
    return hobak_batch_set_pin_targets(_handle, 0, t.data()) == HOBAK_OK;
  }
  bool build() {
    const auto& rest = _tetMesh.restVertices();
    const auto& tets = _tetMesh.tets();
    std::vector<REAL> restFlat(3 * rest.size());
    for (size_t x = 0; x < rest.size(); x++)
      for (int i = 0; i < 3; i++) restFlat[3 * x + i] = rest[x][i];
    std::vector<int> tetFlat(4 * tets.size());
    for (size_t t = 0; t < tets.size(); t++)
      for (int a = 0; a < 4; a++) tetFlat[4 * t + a] = tets[t][a];
    hobak_scene_desc d{};
    d.nv = (int)rest.size();
    d.nt = (int)tets.size();
    d.rest = restFlat.data();
    d.tets = tetFlat.data();
    d.material = _hyperelastic.descriptor();
    d.density = _massScale;
    d.gravity[0] = d.gravity[1] = d.gravity[2] = 0.0;  // external forces are uploaded each solve
    d.dt = _dt;
    d.npinned = (int)_pinned.size();
    d.pinned = _pinned.empty() ? nullptr : _pinned.data();
    _pinnedAt.resize(3 * _pinned.size());
    for (size_t k = 0; k < _pinned.size(); k++)
      for (int i = 0; i < 3; i++) _pinnedAt[3 * k + i] = _position[3 * (size_t)_pinned[k] + i];
    d.x0 = _position.data();
    d.v0 = _velocity.data();
    if (hobak_gpu_create(&d, &_opts, &_handle) != HOBAK_OK) {
      _handle = nullptr;
      return fail();
    }
    return true;
  }
  bool fail() {
    _error = hobak_last_error();
    return false;
  }

  TET_MESH& _tetMesh;
  VOLUME::HYPERELASTIC& _hyperelastic;
  VECTOR _position, _velocity, _externalForces;
  std::vector<int> _pinned;
  std::map<int, std::function<VECTOR3()>> _shapePins;  // pins that follow a shape
  std::vector<REAL> _pinnedAt;                         // pin displacements when built
  REAL _dt = 1.0 / 60.0;  // BACKWARD_EULER_VELOCITY.cpp:37
  REAL _massScale = 1.0;
  REAL _time = 0.0;
  int _currentTimestep = 0;
  std::string _name = "BACKWARD_EULER_VELOCITY";
  hobak_solver_opts _opts{};
  hobak_step_stats _stats{};
  hobak_batch _handle = nullptr;
  std::string _error;
};

// GPU drop-in for BACKWARD_EULER_POSITION (Rayleigh damped,
// BACKWARD_EULER_POSITION.cpp:138-330): the same host-state semantics; the
// unknown of the solve is the position update, and C = alpha M + beta K at
// rest.  Vertex-face and edge-edge contact as in the reference
// (BACKWARD_EULER_POSITION.cpp:187-208).
class BACKWARD_EULER_POSITION : public BACKWARD_EULER_VELOCITY {
 public:
  BACKWARD_EULER_POSITION(TET_MESH& tetMesh, VOLUME::HYPERELASTIC& hyperelastic)
      : BACKWARD_EULER_VELOCITY(tetMesh, hyperelastic) {
    _opts.integrator = HOBAK_INTEGRATOR_POSITION;
    _opts.rayleigh_alpha = 0.01;  // BACKWARD_EULER_POSITION.cpp:53-54
    _opts.rayleigh_beta = 0.01;
    _name = "BACKWARD_EULER_POSITION";
  }
  REAL rayleighAlpha() const { return _opts.rayleigh_alpha; }
  REAL rayleighBeta() const { return _opts.rayleigh_beta; }
  // frozen at the first solve(), like the other settings
  void setRayleigh(const REAL alpha, const REAL beta) {
    _opts.rayleigh_alpha = alpha;
    _opts.rayleigh_beta = beta;
  }
};

// GPU drop-in for NEWMARK (Rayleigh-damped solve, NEWMARK.cpp:183-340): a
// Newton loop of at most maxNewtonIterations() solves on the device;
// acceleration() is host state like position() and velocity().  Contact is
// detected and answered at every Newton iterate (NEWMARK.cpp:226-242).
class NEWMARK : public BACKWARD_EULER_VELOCITY {
 public:
  NEWMARK(TET_MESH& tetMesh, VOLUME::HYPERELASTIC& hyperelastic) : BACKWARD_EULER_VELOCITY(tetMesh, hyperelastic) {
    _opts.integrator = HOBAK_INTEGRATOR_NEWMARK;
    _name = "NEWMARK";
    _acceleration.assign(tetMesh.DOFs(), 0.0);
  }
  // NEWMARK(tetMesh, hyperelastic, damping): the energy-damped solve
  // (NEWMARK.cpp:344-420) with GREEN_DAMPING(mu)
  NEWMARK(TET_MESH& tetMesh, VOLUME::HYPERELASTIC& hyperelastic, const VOLUME::GREEN_DAMPING& damping)
      : NEWMARK(tetMesh, hyperelastic) {
    _greenMu = damping.mu();
  }
  VECTOR& acceleration() { return _acceleration; }
  int& maxNewtonIterations() { return _opts.max_newton; }
  bool solve(const bool verbose) {
    if (!_handle) {
      if (!build()) return false;
      if (_greenMu > 0.0 && hobak_batch_set_green_damping(_handle, 0, _greenMu) != HOBAK_OK) return fail();
    }
    if (hobak_batch_set_acceleration(_handle, 0, _acceleration.data()) != HOBAK_OK) return fail();
    if (!BACKWARD_EULER_VELOCITY::solve(verbose)) return false;
    if (hobak_batch_get_acceleration(_handle, 0, _acceleration.data()) != HOBAK_OK) return fail();
    return true;
  }

 private:
  VECTOR _acceleration;
  REAL _greenMu = 0.0;
};

}  // namespace TIMESTEPPER
}  // namespace HOBAK_GPU
