// Driver around the UNMODIFIED reference (HOBAK) sources, compiled in place by
// oracle/ref/Makefile into oracle/_ref/.  Test infrastructure only: it
// produces golden vectors (tests/golden/) and validates the CPU restatement
// in oracle/.  It never ships and is never linked by the product library.
//
// Modes (all inputs/outputs are .npy files in a directory):
//   elements <in> <out> <material> <mu> <lambda>
//       per-tet F, svd_rv(F), psi, PK1, clampedHessian, hessian, element forces and
//       12x12 Hessians, plus the assembled R and CSC K
//       (TET_MESH.cpp:643-770, TET_MESH_FASTER.cpp:89-133).  Anisotropic
//       materials (aniso_arap, aniso_stvk, aniso_fung, aniso_dirichlet) take
//       their fibre direction from <in>/fiber.npy (run mode too).
//   run <in> <out> <material> <mu> <lambda> <steps> <stride>
//       BACKWARD_EULER_VELOCITY::solve (Timestepper/BACKWARD_EULER_VELOCITY.cpp:96-235)
//       or BACKWARD_EULER_POSITION::solve (Timestepper/BACKWARD_EULER_POSITION.cpp:129-330)
//       for `steps` steps, recording the displacement and velocity every
//       `stride` steps.  Options come from <in>/params.npy:
//         [density, gx, gy, gz, dt, tol, maxit, vf_on, ee_on, coll_eps, coll_mu, coll_beta
//          (, integrator: 0 velocity / 1 position / 2 Newmark, rayleigh_alpha, rayleigh_beta)]
//       NEWMARK::solve (Timestepper/NEWMARK.cpp:183-340) is integrator 2.
//   collide <in> <out> <coll_eps>
//       vertex-face detection at the displacement in <in>/x.npy
//       (TET_MESH_FASTER.cpp:248-334, TET_MESH.cpp:1785-1826).
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <iostream>
#include <memory>
#include <string>
#include <type_traits>
#include <vector>

#include "SETTINGS.h"
#include "Geometry/CUBE.h"
#include "Damping/Volume/GREEN_DAMPING.h"
#include "Geometry/TET_MESH_FASTER.h"
#include "Hyperelastic/Volume/ANISOTROPIC_ARAP.h"
#include "Hyperelastic/Volume/ANISOTROPIC_DIRICHLET.h"
#include "Hyperelastic/Volume/ANISOTROPIC_FUNG.h"
#include "Hyperelastic/Volume/ANISOTROPIC_STVK.h"
#include "Hyperelastic/Volume/ARAP.h"
#include "Hyperelastic/Volume/LINEAR.h"
#include "Hyperelastic/Volume/NEO_HOOKEAN_BW.h"
#include "Hyperelastic/Volume/SNH.h"
#include "Hyperelastic/Volume/SNH_WITH_BARRIER.h"
#include "Hyperelastic/Volume/STVK.h"
#include "Timestepper/BACKWARD_EULER_POSITION.h"
#include "Timestepper/BACKWARD_EULER_VELOCITY.h"
#include "Timestepper/NEWMARK.h"
#include "util/MATRIX_UTIL.h"
#include "npy.h"

using namespace HOBAK;

namespace {

// exposes the protected per-tet caches of the reference mesh
class HarnessMesh : public TET_MESH_FASTER {
 public:
  HarnessMesh(const std::vector<VECTOR3>& rest, const std::vector<VECTOR4I>& tets)
      : TET_MESH_FASTER(rest, tets) {}
  const std::vector<MATRIX9x12>& pFpxs() const { return _pFpxs; }
  const std::vector<REAL>& restVolumes() const { return _restTetVolumes; }
  const std::vector<MATRIX3>& Fs() const { return _Fs; }
  const std::vector<MATRIX3>& Us() const { return _Us; }
  const std::vector<MATRIX3>& Vs() const { return _Vs; }
  const std::vector<VECTOR3>& Sigmas() const { return _Sigmas; }
  const std::vector<MATRIX3>& DmInvs() const { return _DmInvs; }
};

// exposes the protected CG solver settings and pin list of the reference stepper
class HarnessBEV : public TIMESTEPPER::BACKWARD_EULER_VELOCITY {
 public:
  HarnessBEV(TET_MESH& m, VOLUME::HYPERELASTIC& h) : BACKWARD_EULER_VELOCITY(m, h) {}
  void setSolver(double tol, int maxit) {
    _cgSolver.setTolerance(tol);
    _cgSolver.setMaxIterations(maxit);
  }
  int lastIterations() const { return (int)_cgSolver.iterations(); }
  double lastError() const { return (double)_cgSolver.error(); }
  // pin a vertex at its current world position through an identity-transform shape
  void pin(const KINEMATIC_SHAPE* shape, int vertexID, const VECTOR3& world) {
    KINEMATIC_CONSTRAINT c;
    c.shape = shape;
    c.vertexID = vertexID;
    c.localPosition = shape->worldVertexToLocal(world);
    _kinematicConstraints.push_back(c);
  }
};

// the same for the position-based stepper, with its Rayleigh coefficients
class HarnessBEP : public TIMESTEPPER::BACKWARD_EULER_POSITION {
 public:
  HarnessBEP(TET_MESH& m, VOLUME::HYPERELASTIC& h) : BACKWARD_EULER_POSITION(m, h) {}
  void setRayleigh(double alpha, double beta) {
    _rayleighAlpha = alpha;
    _rayleighBeta = beta;
  }
  void setSolver(double tol, int maxit) {
    _cgSolver.setTolerance(tol);
    _cgSolver.setMaxIterations(maxit);
  }
  int lastIterations() const { return (int)_cgSolver.iterations(); }
  double lastError() const { return (double)_cgSolver.error(); }
  void pin(const KINEMATIC_SHAPE* shape, int vertexID, const VECTOR3& world) {
    KINEMATIC_CONSTRAINT c;
    c.shape = shape;
    c.vertexID = vertexID;
    c.localPosition = shape->worldVertexToLocal(world);
    _kinematicConstraints.push_back(c);
  }
};

// and for NEWMARK
class HarnessNewmark : public TIMESTEPPER::NEWMARK {
 public:
  HarnessNewmark(TET_MESH& m, VOLUME::HYPERELASTIC& h) : NEWMARK(m, h) {}
  ~HarnessNewmark() { delete _green; }
  // the energy-damped solve (NEWMARK::solve takes it when _damping is set)
  void setGreenDamping(double mu) {
    delete _green;
    _green = new VOLUME::GREEN_DAMPING(mu);
    _damping = _green;
  }
  VOLUME::GREEN_DAMPING* _green = nullptr;
  void setSolver(double tol, int maxit) {
    _cgSolver.setTolerance(tol);
    _cgSolver.setMaxIterations(maxit);
  }
  int lastIterations() const { return (int)_cgSolver.iterations(); }
  double lastError() const { return (double)_cgSolver.error(); }
  void pin(const KINEMATIC_SHAPE* shape, int vertexID, const VECTOR3& world) {
    KINEMATIC_CONSTRAINT c;
    c.shape = shape;
    c.vertexID = vertexID;
    c.localPosition = shape->worldVertexToLocal(world);
    _kinematicConstraints.push_back(c);
  }
};

// fibre direction of the anisotropic energies: <in>/fiber.npy (3 doubles), else x
VECTOR3 loadFiber(const std::string& dir) {
  FILE* f = std::fopen((dir + "/fiber.npy").c_str(), "rb");
  if (!f) return VECTOR3(1, 0, 0);
  std::fclose(f);
  npy::Array a = npy::load(dir + "/fiber.npy");
  return VECTOR3(a.f8()[0], a.f8()[1], a.f8()[2]);
}

std::unique_ptr<VOLUME::HYPERELASTIC> makeMaterial(const std::string& name, double mu, double lambda,
                                                   const VECTOR3& fiber = VECTOR3(1, 0, 0)) {
  if (name == "aniso_arap") return std::make_unique<VOLUME::ANISOTROPIC_ARAP>(mu, fiber);
  if (name == "aniso_stvk") return std::make_unique<VOLUME::ANISOTROPIC_STVK>(mu, fiber);
  if (name == "aniso_fung") return std::make_unique<VOLUME::ANISOTROPIC_FUNG>(mu, fiber);
  if (name == "aniso_dirichlet") return std::make_unique<VOLUME::ANISOTROPIC_DIRICHLET>(mu, fiber);
  if (name == "snh") return std::make_unique<VOLUME::SNH>(mu, lambda);
  if (name == "arap") return std::make_unique<VOLUME::ARAP>(mu, lambda);
  if (name == "stvk") return std::make_unique<VOLUME::STVK>(mu, lambda);
  if (name == "linear") return std::make_unique<VOLUME::LINEAR>(mu, lambda);
  if (name == "neo_hookean_bw") return std::make_unique<VOLUME::NEO_HOOKEAN_BW>(mu, lambda);
  if (name == "snh_barrier") return std::make_unique<VOLUME::SNH_WITH_BARRIER>(mu, lambda);
  throw std::runtime_error("unknown material " + name);
}

void loadMesh(const std::string& dir, std::vector<VECTOR3>& rest, std::vector<VECTOR4I>& tets) {
  npy::Array r = npy::load(dir + "/rest.npy"), t = npy::load(dir + "/tets.npy");
  rest.resize(r.shape[0]);
  for (long i = 0; i < r.shape[0]; i++) rest[i] = VECTOR3(r.f8()[3 * i], r.f8()[3 * i + 1], r.f8()[3 * i + 2]);
  tets.resize(t.shape[0]);
  for (long i = 0; i < t.shape[0]; i++)
    tets[i] = VECTOR4I(t.i4()[4 * i], t.i4()[4 * i + 1], t.i4()[4 * i + 2], t.i4()[4 * i + 3]);
}

VECTOR loadVector(const std::string& path, long n) {
  npy::Array a = npy::load(path);
  if (a.size() != n) throw std::runtime_error("size mismatch in " + path);
  VECTOR v(n);
  for (long i = 0; i < n; i++) v[i] = a.f8()[i];
  return v;
}

void save3(const std::string& path, const std::vector<MATRIX3>& Ms) {
  std::vector<double> buf(9 * Ms.size());
  for (size_t i = 0; i < Ms.size(); i++) {
    const VECTOR9 f = flatten(Ms[i]);
    for (int k = 0; k < 9; k++) buf[9 * i + k] = f[k];
  }
  npy::save(path, buf.data(), "<f8", {(long)Ms.size(), 9});
}

int modeElements(const std::string& in, const std::string& out, const std::string& mat, double mu, double lambda) {
  std::vector<VECTOR3> rest;
  std::vector<VECTOR4I> tets;
  loadMesh(in, rest, tets);
  const long nv = rest.size(), nt = tets.size();
  HarnessMesh mesh(rest, tets);
  auto material = makeMaterial(mat, mu, lambda, loadFiber(in));
  mesh.setDisplacement(loadVector(in + "/x.npy", 3 * nv));
  mesh.computeFs();
  mesh.computeSVDs();

  save3(out + "/F.npy", mesh.Fs());
  save3(out + "/U.npy", mesh.Us());
  save3(out + "/V.npy", mesh.Vs());
  save3(out + "/DmInv.npy", mesh.DmInvs());
  std::vector<double> sig(3 * nt), psi(nt), P(9 * nt), H9(81 * nt), H9u(81 * nt), fe(12 * nt), H12(144 * nt),
      vol(nt);
  for (long i = 0; i < nt; i++) {
    const MATRIX3& F = mesh.Fs()[i];
    for (int k = 0; k < 3; k++) sig[3 * i + k] = mesh.Sigmas()[i][k];
    psi[i] = material->psi(F);
    vol[i] = mesh.restVolumes()[i];
    const MATRIX3 PK1 = material->PK1(F);
    const VECTOR9 pf = flatten(PK1);
    for (int k = 0; k < 9; k++) P[9 * i + k] = pf[k];
    const MATRIX9 H = material->clampedHessian(mesh.Us()[i], mesh.Sigmas()[i], mesh.Vs()[i]);
    for (int c = 0; c < 9; c++)
      for (int r = 0; r < 9; r++) H9[81 * i + 9 * c + r] = H(r, c);  // column-major
    const MATRIX9 Hu = material->hessian(F);  // unclamped (HYPERELASTIC.h:44)
    for (int c = 0; c < 9; c++)
      for (int r = 0; r < 9; r++) H9u[81 * i + 9 * c + r] = Hu(r, c);
    const MATRIX9x12& pFpx = mesh.pFpxs()[i];
    const VECTOR12 f = -vol[i] * (pFpx.transpose() * pf);
    for (int k = 0; k < 12; k++) fe[12 * i + k] = f[k];
    const MATRIX12 He = (pFpx.transpose() * (-vol[i] * H)) * pFpx;
    for (int c = 0; c < 12; c++)
      for (int r = 0; r < 12; r++) H12[144 * i + 12 * c + r] = He(r, c);
  }
  npy::save(out + "/Sigma.npy", sig.data(), "<f8", {nt, 3});
  npy::save(out + "/psi.npy", psi.data(), "<f8", {nt});
  npy::save(out + "/P.npy", P.data(), "<f8", {nt, 9});
  npy::save(out + "/H9.npy", H9.data(), "<f8", {nt, 81});
  npy::save(out + "/H9u.npy", H9u.data(), "<f8", {nt, 81});
  npy::save(out + "/fe.npy", fe.data(), "<f8", {nt, 12});
  npy::save(out + "/He.npy", H12.data(), "<f8", {nt, 144});
  npy::save(out + "/restVolume.npy", vol.data(), "<f8", {nt});
  std::vector<double> orv(mesh.restOneRingVolumes().begin(), mesh.restOneRingVolumes().end());
  npy::save(out + "/oneRingVolume.npy", orv.data(), "<f8", {nv});

  const VECTOR R = mesh.computeHyperelasticForces(*material);
  npy::save(out + "/R.npy", R.data(), "<f8", {3 * nv});
  double energy = mesh.computeHyperelasticEnergy(*material);
  npy::save(out + "/energy.npy", &energy, "<f8", {1});

  SPARSE_MATRIX K = mesh.computeHyperelasticClampedHessian(*material);
  K.makeCompressed();
  std::vector<int32_t> colptr(K.outerIndexPtr(), K.outerIndexPtr() + K.outerSize() + 1);
  std::vector<int32_t> rowidx(K.innerIndexPtr(), K.innerIndexPtr() + K.nonZeros());
  npy::save(out + "/K_colptr.npy", colptr.data(), "<i4", {(long)colptr.size()});
  npy::save(out + "/K_rowidx.npy", rowidx.data(), "<i4", {(long)rowidx.size()});
  npy::save(out + "/K_values.npy", K.valuePtr(), "<f8", {(long)K.nonZeros()});
  return 0;
}

template <class Stepper>
int runWith(const std::string& in, const std::string& out, const std::string& mat, double mu, double lambda,
            int steps, int stride) {
  std::vector<VECTOR3> rest;
  std::vector<VECTOR4I> tets;
  loadMesh(in, rest, tets);
  const long nv = rest.size();
  npy::Array prm = npy::load(in + "/params.npy");
  const double* p = prm.f8();
  const long nprm = prm.size();
  const double density = p[0];
  const VECTOR3 gravity(p[1], p[2], p[3]);
  const double dt = p[4], tol = p[5];
  const int maxit = (int)p[6];
  const bool vf = p[7] != 0.0, ee = p[8] != 0.0;
  const double collEps = p[9], collMu = p[10], collBeta = p[11];

  HarnessMesh mesh(rest, tets);
  if (vf || ee) mesh.setCollisionEps(collEps);
  auto material = makeMaterial(mat, mu, lambda, loadFiber(in));
  const VECTOR x0 = loadVector(in + "/x0.npy", 3 * nv);
  const VECTOR v0 = loadVector(in + "/v0.npy", 3 * nv);
  npy::Array pins = npy::load(in + "/pinned.npy");

  Stepper solver(mesh, *material);
  if constexpr (std::is_same_v<Stepper, HarnessBEP>) {
    if (nprm >= 15) solver.setRayleigh(p[13], p[14]);
  }
  if constexpr (std::is_same_v<Stepper, HarnessNewmark>) {
    if (nprm >= 16 && p[15] > 0.0) solver.setGreenDamping(p[15]);
  }
  solver.setDt(dt);
  solver.setSolver(tol, maxit);
  solver.vertexFaceSelfCollisionsOn() = vf;
  solver.edgeEdgeSelfCollisionsOn() = ee;
  solver.collisionStiffness() = collMu;
  solver.collisionDampingBeta() = collBeta;
  solver.scaleMass(density);

  // deformed start: pins are attached in the deformed state
  mesh.setDisplacement(x0);
  CUBE identity(VECTOR3(0, 0, 0), 1.0);
  for (long i = 0; i < pins.size(); i++) {
    const int v = pins.i4()[i];
    solver.pin(&identity, v, mesh.vertices()[v]);
  }
  solver.position() = x0;
  solver.velocity() = v0;

  const int nrec = steps / stride + 1;
  std::vector<double> xs(nrec * 3 * nv), vs(nrec * 3 * nv), ms(steps);
  std::vector<int32_t> iters(steps);
  std::vector<double> errs(steps);
  auto record = [&](int slot) {
    for (long k = 0; k < 3 * nv; k++) {
      xs[slot * 3 * nv + k] = solver.position()[k];
      vs[slot * 3 * nv + k] = solver.velocity()[k];
    }
  };
  record(0);
  for (int s = 0; s < steps; s++) {
    solver.externalForces().setZero();
    solver.addGravity(density * gravity);
    auto t0 = std::chrono::steady_clock::now();
    solver.solve(false);
    auto t1 = std::chrono::steady_clock::now();
    ms[s] = std::chrono::duration<double, std::milli>(t1 - t0).count();
    iters[s] = solver.lastIterations();
    errs[s] = solver.lastError();
    if ((s + 1) % stride == 0) record((s + 1) / stride);
  }
  npy::save(out + "/x.npy", xs.data(), "<f8", {nrec, 3 * nv});
  npy::save(out + "/v.npy", vs.data(), "<f8", {nrec, 3 * nv});
  npy::save(out + "/step_ms.npy", ms.data(), "<f8", {steps});
  npy::save(out + "/iters.npy", iters.data(), "<i4", {steps});
  npy::save(out + "/cg_error.npy", errs.data(), "<f8", {steps});
  double energy = mesh.computeHyperelasticEnergy(*material);
  npy::save(out + "/energy.npy", &energy, "<f8", {1});
  return 0;
}

int modeRun(const std::string& in, const std::string& out, const std::string& mat, double mu, double lambda,
            int steps, int stride) {
  npy::Array prm = npy::load(in + "/params.npy");
  const double integrator = prm.size() >= 13 ? prm.f8()[12] : 0.0;
  if (integrator == 1.0) return runWith<HarnessBEP>(in, out, mat, mu, lambda, steps, stride);
  if (integrator == 2.0) return runWith<HarnessNewmark>(in, out, mat, mu, lambda, steps, stride);
  return runWith<HarnessBEV>(in, out, mat, mu, lambda, steps, stride);
}

int modeCollide(const std::string& in, const std::string& out, double eps) {
  std::vector<VECTOR3> rest;
  std::vector<VECTOR4I> tets;
  loadMesh(in, rest, tets);
  const long nv = rest.size();
  HarnessMesh mesh(rest, tets);
  mesh.setCollisionEps(eps);
  mesh.setDisplacement(loadVector(in + "/x.npy", 3 * nv));
  mesh.computeFs();
  mesh.computeSVDs();
  mesh.refitAABB();
  mesh.computeVertexFaceCollisions();
  const auto& pairs = mesh.vertexFaceCollisions();
  std::vector<int32_t> buf(2 * pairs.size());
  for (size_t i = 0; i < pairs.size(); i++) {
    buf[2 * i] = pairs[i].first;
    buf[2 * i + 1] = pairs[i].second;
  }
  npy::save(out + "/vf_pairs.npy", buf.data(), "<i4", {(long)pairs.size(), 2});
  const auto& tris = mesh.surfaceTriangles();
  std::vector<int32_t> tb(3 * tris.size());
  for (size_t i = 0; i < tris.size(); i++)
    for (int k = 0; k < 3; k++) tb[3 * i + k] = tris[i][k];
  npy::save(out + "/surface_triangles.npy", tb.data(), "<i4", {(long)tris.size(), 3});
  const auto& sv = mesh.surfaceVertices();
  std::vector<int32_t> svb(sv.begin(), sv.end());
  npy::save(out + "/surface_vertices.npy", svb.data(), "<i4", {(long)sv.size()});
  return 0;
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    std::fprintf(stderr, "usage: hobak_ref elements|run|collide ...\n");
    return 2;
  }
  const std::string mode = argv[1];
  try {
    if (mode == "elements" && argc == 7)
      return modeElements(argv[2], argv[3], argv[4], std::atof(argv[5]), std::atof(argv[6]));
    if (mode == "run" && argc == 9)
      return modeRun(argv[2], argv[3], argv[4], std::atof(argv[5]), std::atof(argv[6]), std::atoi(argv[7]),
                     std::atoi(argv[8]));
    if (mode == "collide" && argc == 5) return modeCollide(argv[2], argv[3], std::atof(argv[4]));
  } catch (const std::exception& e) {
    std::fprintf(stderr, "hobak_ref: %s\n", e.what());
    return 1;
  }
  std::fprintf(stderr, "hobak_ref: bad arguments for mode %s\n", mode.c_str());
  return 2;
}
