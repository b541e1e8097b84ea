/*
 * hobak_gpu.h -- C ABI of the GB300 (sm_103a) implicit tet-FEM timestep.
 *
 * A drop-in for HOBAK's BACKWARD_EULER_VELOCITY::solve hot path with its
 * VOLUME::HYPERELASTIC energies.  Plain C types only: host buffers are
 * caller-owned, device buffers are library-owned, handles are opaque.  Every
 * call returns an int status (HOBAK_OK = 0; negative = error; positive =
 * warning) and never throws.  The message of the last failing call on the
 * calling thread is available from hobak_last_error().
 *
 * State conventions follow the reference:
 *   - vectors are interleaved xyz, 3*nv doubles;
 *   - the position state is the DISPLACEMENT from rest, like
 *     TIMESTEPPER::_position (Timestepper/TIMESTEPPER.h:190);
 *   - the mass matrix is diag(density * one-ring volume)
 *     (TIMESTEPPER.cpp:176-208 with scaleMass, TIMESTEPPER.h:100);
 *   - pinned vertices are held at the displacement they had when pinned
 *     (attachKinematicConstraints, TIMESTEPPER.cpp:380-403 with
 *     applyKinematicConstraints, TIMESTEPPER.cpp:105-122).
 */
#ifndef HOBAK_GPU_H
#define HOBAK_GPU_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define HOBAK_OK 0
#define HOBAK_WARN_NOT_CONVERGED 1   /* PCG hit max iterations in some scene */
#define HOBAK_ERR_INVALID -1         /* bad argument, size or handle */
#define HOBAK_ERR_CUDA -2            /* CUDA runtime error (message in hobak_last_error) */
#define HOBAK_ERR_NAN -3             /* non-finite value detected in a solve */
#define HOBAK_ERR_NO_MEMORY -4       /* device allocation failed */
#define HOBAK_ERR_ADMISSION -5       /* serving: job does not fit the memory budget */
#define HOBAK_ERR_TIMEOUT -6         /* a bounded device wait gave up */
#define HOBAK_ERR_NO_DEVICE -7       /* no usable sm_103 device */
#define HOBAK_ERR_OVERFLOW -8        /* a fixed-capacity device list overflowed (collision candidates) */

/* ---- materials: the VOLUME::HYPERELASTIC family (Hyperelastic/Volume/) ---- */
#define HOBAK_MATERIAL_SNH 0            /* SNH.cpp (Stable Neo-Hookean)        */
#define HOBAK_MATERIAL_ARAP 1           /* ARAP.cpp                            */
#define HOBAK_MATERIAL_STVK 2           /* STVK.cpp (St. Venant-Kirchhoff)     */
#define HOBAK_MATERIAL_LINEAR 3         /* LINEAR.cpp                          */
#define HOBAK_MATERIAL_NEO_HOOKEAN_BW 4 /* NEO_HOOKEAN_BW.cpp                  */
#define HOBAK_MATERIAL_SNH_BARRIER 5    /* SNH_WITH_BARRIER.cpp                */
/* anisotropic energies along a fibre direction (hobak_material.fiber) */
#define HOBAK_MATERIAL_ANISOTROPIC_ARAP 6      /* ANISOTROPIC_ARAP.cpp      */
#define HOBAK_MATERIAL_ANISOTROPIC_STVK 7      /* ANISOTROPIC_STVK.cpp      */
#define HOBAK_MATERIAL_ANISOTROPIC_FUNG 8      /* ANISOTROPIC_FUNG.cpp      */
#define HOBAK_MATERIAL_ANISOTROPIC_DIRICHLET 9 /* ANISOTROPIC_DIRICHLET.cpp */

/* ---- precision modes ---- */
#define HOBAK_PRECISION_FP64 0   /* every kernel in FP64 */
#define HOBAK_PRECISION_MIXED 1  /* FP32 Hessian/SpMV/inner PCG, FP64 SVD, residual and refinement */

/* ---- preconditioners ---- */
#define HOBAK_INTEGRATOR_VELOCITY 0   /* BACKWARD_EULER_VELOCITY::solve (BACKWARD_EULER_VELOCITY.cpp:96-235) */
#define HOBAK_INTEGRATOR_POSITION 1   /* BACKWARD_EULER_POSITION::solveRayleighDamped (BACKWARD_EULER_POSITION.cpp:138-330) */
#define HOBAK_INTEGRATOR_NEWMARK 2    /* NEWMARK::solveRayleighDamped (NEWMARK.cpp:183-340): a Newton loop */

#define HOBAK_PRECOND_JACOBI 0        /* scalar 1/diag, Eigen DiagonalPreconditioner */
#define HOBAK_PRECOND_BLOCK_JACOBI 1  /* inverse of each 3x3 diagonal block */

/* Lame parameters as the reference materials take them: the constructor
 * arguments (mu, lambda) of SNH(mu, lambda), ARAP(mu, lambda), ...  The SNH
 * reparameterisation lambda' = lambda + mu (SNH.cpp:23-32) happens inside.
 * The anisotropic energies take (mu, a): ANISOTROPIC_ARAP(mu, a) and its
 * siblings (ANISOTROPIC_ARAP.h:28); lambda is unused there and `fiber` is a,
 * normalised inside as their constructors do (ANISOTROPIC_ARAP.cpp:26-29). */
typedef struct hobak_material {
  int kind;      /* HOBAK_MATERIAL_* */
  double mu;
  double lambda;
  double fiber[3];  /* anisotropic energies only: the fibre direction a */
} hobak_material;

/* One scene (one tet mesh with its material and pins). */
typedef struct hobak_scene_desc {
  int nv;                  /* vertices */
  int nt;                  /* tets */
  const double* rest;      /* 3*nv rest positions */
  const int* tets;         /* 4*nt vertex ids, positive rest volume */
  hobak_material material;
  double density;          /* mass scale: M = density * diag(one-ring volume) */
  double gravity[3];       /* body force per unit mass; f_ext = M g per vertex */
  double dt;               /* time step (reference default 1/60, BEV.cpp:37) */
  int npinned;
  const int* pinned;       /* pinned vertex ids (may be NULL if npinned == 0) */
  const double* x0;        /* 3*nv initial displacement (NULL = zero); pins take x0 */
  const double* v0;        /* 3*nv initial velocity (NULL = zero) */
} hobak_scene_desc;

/* Linear solver options (Eigen ConjugateGradient equivalents,
 * ext/eigen-3.3.7/Eigen/src/IterativeLinearSolvers/ConjugateGradient.h). */
typedef struct hobak_solver_opts {
  double tol;              /* relative residual: stop when |r| < tol |rhs| */
  int max_iters;           /* per solve */
  int precision;           /* HOBAK_PRECISION_* */
  int preconditioner;      /* HOBAK_PRECOND_* */
  int max_refinements;     /* MIXED only: FP64 iterative-refinement sweeps (<= 3) */
  int use_graph;           /* capture each step as a CUDA graph (1) or launch eagerly (0) */
  int integrator;          /* HOBAK_INTEGRATOR_* (default VELOCITY) */
  double rayleigh_alpha;   /* POSITION: C = alpha M + beta K(rest) (defaults 0.01, 0.01: */
  double rayleigh_beta;    /*   BACKWARD_EULER_POSITION.cpp:53-54) */
  int max_newton;          /* NEWMARK: Newton iterations per step at most (default 10) */
  double newton_tolerance; /* NEWMARK: stop once |rhs|^2 <= this (default 1e-7, NEWMARK.cpp:43) */
  double inner_tolerance;  /* MIXED: each FP32 inner solve stops at this relative residual at the
                              tightest (default 1e-5; the FP64 test on the outer residual is unchanged) */
} hobak_solver_opts;

/* Per-scene statistics of the last step. */
typedef struct hobak_step_stats {
  int iterations;          /* PCG iterations of the last step (summed over refinement sweeps) */
  int converged;           /* 1 when the residual test passed */
  double rel_residual;     /* sqrt(|r|^2 / |rhs|^2) at exit (Eigen's error()) */
  int refinements;         /* MIXED: refinement sweeps used */
} hobak_step_stats;

typedef struct hobak_batch_t* hobak_batch;

/* Library version and device check. */
const char* hobak_version(void);
const char* hobak_last_error(void);
int hobak_device_check(int* sm_major, int* sm_minor, int* num_sms);

/* Default options: tol 1e-8, 1000 iterations, FP64, block Jacobi, 3 refinements, graph on. */
void hobak_default_solver_opts(hobak_solver_opts* opts);

/* ---- batched API: many scenes packed into one device-resident batch ----
 * Replaces one BACKWARD_EULER_VELOCITY per scene (BACKWARD_EULER_VELOCITY.cpp:31-46)
 * with all scenes stepped together; each scene's result does not depend on
 * the others (per-scene reductions, no cross-scene atomics). */
int hobak_batch_create(const hobak_scene_desc* scenes, int nscenes, const hobak_solver_opts* opts,
                       hobak_batch* out);
int hobak_batch_destroy(hobak_batch b);
int hobak_batch_num_scenes(hobak_batch b, int* n);
/* Advance every scene by nsteps BACKWARD_EULER_VELOCITY::solve steps
 * (BACKWARD_EULER_VELOCITY.cpp:96-235).  State stays on the device.
 * stats may be NULL or point at nscenes entries (stats of the last step). */
int hobak_batch_step(hobak_batch b, int nsteps, hobak_step_stats* stats);
/* hobak_batch_step split in two (no reference counterpart; for overlapping
 * several batches on the device): enqueue nsteps steps and return at once,
 * then wait for them and collect the stats of the last step. */
int hobak_batch_step_async(hobak_batch b, int nsteps);
int hobak_batch_wait(hobak_batch b, hobak_step_stats* stats);
/* Non-blocking: 1 when everything enqueued on the batch has finished (a
 * following hobak_batch_wait returns without blocking), 0 while work is still
 * running, negative on error. */
int hobak_batch_query(hobak_batch b);
/* Park (active = 0) or resume one scene: a parked scene keeps its state and is
 * skipped by every kernel, so a serving loop can retire finished jobs without
 * re-packing the batch (no reference counterpart). */
int hobak_batch_set_active(hobak_batch b, int scene, int active);
/* Host <-> device state of one scene (3*nv doubles each; NULL skips). */
int hobak_batch_set_state(hobak_batch b, int scene, const double* x, const double* v);
int hobak_batch_get_state(hobak_batch b, int scene, double* x, double* v);
/* NEWMARK's acceleration state of one scene (3*nv, zero at creation; the
 * other integrators leave it untouched). */
int hobak_batch_get_acceleration(hobak_batch b, int scene, double* a);
int hobak_batch_set_acceleration(hobak_batch b, int scene, const double* a);
/* NEWMARK's energy-damped solve for one scene: the damping of
 * NEWMARK(mesh, material, GREEN_DAMPING(mu)) (NEWMARK.h constructor with a
 * DAMPING; NEWMARK::solveEnergyDamped, NEWMARK.cpp:344-420;
 * GREEN_DAMPING.cpp:46-50).  mu = 0 turns it off.  NEWMARK batches only: the
 * reference's damped BACKWARD_EULER_VELOCITY solve reads a never-computed
 * Fdot, so other integrators refuse it. */
int hobak_batch_set_green_damping(hobak_batch b, int scene, double mu);
/* Move one scene's pins: 3 target displacements (world - rest) per pinned
 * vertex, in the order hobak_scene_desc.pinned listed them.  Replaces
 * applyKinematicConstraints recomputing the targets from moved kinematic
 * shapes at the start of each solve (TIMESTEPPER.cpp:105-122; scenes such as
 * NEWMARK_STRETCH.h move a shape between frames).  Applies from the next step. */
int hobak_batch_set_pin_targets(hobak_batch b, int scene, const double* targets);
/* Snapshot of the batch's dynamic state (x, v, acceleration, external forces,
 * pin targets, active flags) into host or device memory, and back.  The
 * reference's counterpart is the per-frame JSON record of position, velocity
 * and external forces (FILE_IO.cpp:427-445); a snapshot restores a batch with
 * the same scenes bitwise.  snapshot_bytes gives the size; dst/src may be any
 * host or device pointer; restore refuses a snapshot of other scenes. */
int hobak_batch_snapshot_bytes(hobak_batch b, size_t* bytes);
int hobak_batch_snapshot(hobak_batch b, void* dst, size_t bytes);
int hobak_batch_restore(hobak_batch b, const void* src, size_t bytes);
/* Whole batch at once: every scene's 3*nv values back to back in scene
 * order (total 3 * sum(nv)); one copy each.  The set calls are enqueued on
 * the batch's stream and return at once: host buffers must stay unchanged
 * until the next step, wait or get call returns (pageable buffers are copied
 * before return).  get_state_all returns with the data on the host. */
int hobak_batch_set_state_all(hobak_batch b, const double* x, const double* v);
int hobak_batch_get_state_all(hobak_batch b, double* x, double* v);
int hobak_batch_set_external_forces_all(hobak_batch b, const double* f);
/* Replace the external force vector (3*nv) of one scene; the default is M g. */
int hobak_batch_set_external_forces(hobak_batch b, int scene, const double* f);
int hobak_batch_set_solver(hobak_batch b, const hobak_solver_opts* opts);
/* Vertex-face self collisions of one scene (TIMESTEPPER's
 * vertexFaceSelfCollisionsOn / collisionStiffness / collisionDampingBeta,
 * TIMESTEPPER.h:62-69, and TET_MESH::setCollisionEps, TET_MESH.cpp:2160-2165).
 * Off by default here; the reference turns vertex-face and edge-edge self
 * collisions on by default (TIMESTEPPER.cpp:83-84), so a binding that mirrors
 * a stock HOBAK timestepper also calls hobak_batch_set_edge_collisions
 * (hobak_gpu_set_edge_collisions).  Detection runs on the GPU every step: a spatial hash replaces
 * the AABB tree, the narrow phase is the reference's
 * (TET_MESH_FASTER.cpp:248-334).  The first call builds the surfaces of every
 * scene in the batch. */
int hobak_batch_set_collisions(hobak_batch b, int scene, int vf_on, double eps, double stiffness,
                               double damping_beta);
/* Edge-edge self collisions of one scene on or off (TIMESTEPPER's
 * edgeEdgeSelfCollisionsOn, TIMESTEPPER.h:62-69): surface edge pairs
 * (TET_MESH_FASTER::computeEdgeEdgeCollisions, TET_MESH_FASTER.cpp:340-500)
 * with EDGE_SQRT_COLLISION forces and clamped Hessians, using the collision
 * distance, stiffness and damping set with hobak_batch_set_collisions (the
 * reference's defaults 0.01, 1, 0.001 when never set).  Every integrator
 * (NEWMARK: at every Newton iterate, NEWMARK.cpp:226-242); off by default. */
int hobak_batch_set_edge_collisions(hobak_batch b, int scene, int ee_on);
/* The edge-edge pairs of the last detection as scene-local vertex quadruples
 * (edge0[0], edge0[1], edge1[0], edge1[1]), in surface edge order; *npairs
 * gets the count, at most cap quadruples are written (quads may be NULL). */
int hobak_batch_edge_pairs(hobak_batch b, int scene, int* npairs, int* quads, int cap);
/* Vertex-face pairs of one scene found by the last step's detection (or by a
 * fresh detection at the current state when `detect_now` is 1): *npairs is
 * the count; up to cap (vertex, surface triangle) pairs in scene-local ids,
 * sorted.  Surface triangles (3 ints each, scene-local vertex ids, reference
 * order and winding) when tris is not NULL. */
int hobak_batch_collision_pairs(hobak_batch b, int scene, int detect_now, int* npairs, int* pairs, int cap,
                                int* ntris, int* tris);
/* Per-pair response of the last detection, in the order of
 * hobak_batch_collision_pairs: collision tet (4 scene-local vertex ids:
 * vertex, face[2], face[1], face[0]; TET_MESH.cpp:1785-1826), force
 * -w grad psi (12) and clamped Hessian -w H+ (144, column major)
 * (TET_MESH.cpp:1831-1877, 2045-2088).  Any output may be NULL. */
int hobak_batch_collision_response(hobak_batch b, int scene, int cap, int* tets, double* force, double* hessian);
/* Device memory held by the batch, in bytes. */
int hobak_batch_device_bytes(hobak_batch b, long long* bytes);
/* Mesh-wide hyperelastic energy sum(restVolume * psi(F)) of one scene
 * (TET_MESH::computeHyperelasticEnergy, TET_MESH.cpp:719-731). */
int hobak_batch_energy(hobak_batch b, int scene, double* energy);

/* ---- single-scene API: the BACKWARD_EULER_VELOCITY drop-in ----
 * A batch of one.  hobak_gpu_step uploads nothing and downloads nothing;
 * pair it with set/get_state for host-side state like the reference's
 * position()/velocity() references (TIMESTEPPER.h:53-58). */
int hobak_gpu_create(const hobak_scene_desc* scene, const hobak_solver_opts* opts, hobak_batch* out);
int hobak_gpu_step(hobak_batch b, int nsteps, hobak_step_stats* stats);
int hobak_gpu_set_state(hobak_batch b, const double* x, const double* v);
int hobak_gpu_get_state(hobak_batch b, double* x, double* v);
/* TIMESTEPPER::externalForces() (TIMESTEPPER.h:58), 3*nv doubles. */
int hobak_gpu_set_external_forces(hobak_batch b, const double* f);
/* vertexFaceSelfCollisionsOn(), TET_MESH::setCollisionEps, collisionStiffness(),
 * collisionDampingBeta() (TIMESTEPPER.h:62-69; TET_MESH.cpp:2160-2174). */
int hobak_gpu_set_collisions(hobak_batch b, int vf_on, double eps, double stiffness, double damping_beta);
/* edgeEdgeSelfCollisionsOn() (TIMESTEPPER.h:62-69; on by default in the
 * reference, TIMESTEPPER.cpp:84): the single-scene form of
 * hobak_batch_set_edge_collisions. */
int hobak_gpu_set_edge_collisions(hobak_batch b, int ee_on);
/* _cgSolver.setTolerance / setMaxIterations (IterativeSolverBase.h:281-284,
 * 363) plus precision and preconditioner. */
int hobak_gpu_set_solver(hobak_batch b, const hobak_solver_opts* opts);
int hobak_gpu_destroy(hobak_batch b);

/* ---- element-level entry points (the VOLUME::HYPERELASTIC boundary) ----
 * Batched, device-evaluated material and element terms for n deformation
 * gradients / tets.  Host buffers in and out.  Any output may be NULL.
 *   hobak_material_eval: psi(F) (HYPERELASTIC.h:36), PK1(F) (HYPERELASTIC.h:40),
 *     clampedHessian (HYPERELASTIC.h:48), F column major (flatten,
 *     MATRIX_UTIL.cpp:33-43), Hessians 81 per F, column major.
 *   hobak_element_eval: per tet F = Ds DmInv (TET_MESH.cpp:706-714),
 *     rotation-variant SVD (svd_rv, MATRIX_UTIL.cpp:76-95), element force
 *     -V pFpx^T vec(P) (TET_MESH.cpp:736-747) and element Hessian
 *     pFpx^T (-V clampedHessian) pFpx (TET_MESH_FASTER.cpp:95-103), 144 per
 *     tet, column major. */
int hobak_material_eval(const hobak_material* m, int n, const double* F, double* psi, double* P, double* H);
/* hessian(F) (HYPERELASTIC.h:44): the unclamped 9x9 d2psi/dF2 of n
 * gradients, 81 per F, column major. */
int hobak_material_hessian(const hobak_material* m, int n, const double* F, double* H);
/* The (U, Sigma, V) overloads psi, PK1, hessian and clampedHessian
 * (HYPERELASTIC.h:37, 41, 45, 49) for n factorisations (U and V 9 doubles,
 * column major; sigma 3 doubles each, svd_rv convention).  As in the
 * reference, ARAP and the eigensystem-based Hessians use the factors
 * themselves and the F-form energies F = U diag(sigma) V^T.  Any output
 * may be NULL. */
int hobak_material_eval_svd(const hobak_material* m, int n, const double* U, const double* sigma, const double* V,
                            double* psi, double* P, double* H, double* clampedH);
/* energyNeedsSVD() / PK1NeedsSVD() (HYPERELASTIC.h:56-59) of a material kind. */
int hobak_material_needs_svd(int kind, int* energy, int* pk1);
int hobak_element_eval(int nv, int nt, const double* rest, const int* tets, const double* x,
                       const hobak_material* m, double* F, double* sigma, double* force, double* hessian);
/* Assembled stiffness of one scene at its current state: BSR pattern
 * (rowptr nv+1, cols nblocks), K blocks (9 each, column major) and forces R
 * (3*nv).  K and R follow TET_MESH_FASTER::computeHyperelasticClampedHessian
 * (TET_MESH_FASTER.cpp:89-133) and TET_MESH::computeHyperelasticForces
 * (TET_MESH.cpp:736-770).  Call with NULL outputs to query nblocks. */
int hobak_batch_assemble(hobak_batch b, int scene, int* nblocks, int* rowptr, int* cols, double* K, double* R);

/* ---- allocation-free element evaluation (no counterpart in the reference) ----
 * For callers that cannot let a library call cudaMalloc/cudaFree: plugins in
 * hosts that own the device-memory budget, or per-frame loops where an
 * allocation would synchronise the device.  Same results as
 * hobak_element_eval, but every array argument is a DEVICE pointer the caller
 * owns (tets 16-byte aligned), `stream` is a cudaStream_t (NULL = default
 * stream), and the call allocates nothing: its per-tet rest-shape scratch
 * lives in one static device array of HOBAK_NOALLOC_MAX_TETS tets (10 MiB),
 * held by every GPU that loads the library until the process exits.  Larger
 * calls return HOBAK_ERR_INVALID.  The first call on a device looks up that
 * array's address (cudaGetSymbolAddress) and should come before any stream
 * capture.  All calls share the array: calls whose work overlaps on the GPU
 * race and must be serialised by the caller.  Returns once its work on
 * `stream` is done; a tet naming a vertex outside [0, nv) is reported as
 * HOBAK_ERR_INVALID before any element is evaluated. */
#define HOBAK_NOALLOC_MAX_TETS 131072
int hobak_element_eval_noalloc(int nv, int nt, const double* rest, const int* tets, const double* x,
                               const hobak_material* m, double* F, double* sigma, double* force, double* hessian,
                               void* stream);

/* ---- measurement (no reference counterpart; the reference's TIMER,
 * util/TIMER.h:33-76, is replaced by CUDA events) ---- */
/* The CUDA stream (a cudaStream_t) all work of the batch is issued on. */
int hobak_batch_get_stream(hobak_batch b, void** stream);
/* Phase timers: when on, every step records CUDA events around its phases.
 * hobak_batch_phase_times returns, since the last call, the summed ms and the
 * kernel launches of the 5 phases: [element, assembly+preconditioner,
 * rhs+pcg init, pcg iterations, update], then resets them. */
int hobak_batch_enable_timing(hobak_batch b, int on);
int hobak_batch_phase_times(hobak_batch b, double* ms, long long* launches);
/* Kernels launched by this batch since creation. */
int hobak_batch_launch_count(hobak_batch b, long long* launches);
/* Per-launch device time (ms, CUDA events, reps back-to-back launches on the
 * batch stream, at the current state) of the hot kernels
 * [element, assembly, spmv, pcg update], and their algorithmic bytes per
 * launch (every array counted once). */
int hobak_batch_time_kernels(hobak_batch b, int reps, double* ms);
int hobak_batch_kernel_bytes(hobak_batch b, double* bytes);

/* Launch shapes of a batch (no reference counterpart): vertices per PCG tile
 * (64 or 128; one CTA of the SpMV/update/reduction kernels), CTA sizes of the
 * element kernel (64 or 128) and of the assembly kernel (64..1024, multiple of
 * 32), PCG iterations per graph loop body / host poll (1..64), and whether
 * scenes whose vectors fit the shared memory of at most cluster_max CTAs
 * (one vertex per thread, or several in the largest cluster; contact scenes
 * included) solve their linear system inside one thread-block cluster (1;
 * beside the tile path for the others) or on the batch-wide tile path (0,
 * the default), and the largest cluster such a scene may use (cluster_max:
 * 1, 2, 4, 8 or 16 CTAs; larger scenes keep the tile path, which spreads them
 * over the whole GPU).  step_ms is the measured
 * step time of the chosen shape (autotune only; 0 otherwise).  The tile size and
 * the PCG path change results, and only by FP rounding (they change the shape
 * of the dot-product reduction trees). */
typedef struct hobak_tuning {
  int tile_vertices;
  int element_threads;
  int assembly_threads;
  int pcg_chunk;
  int cluster_pcg;
  int cluster_max;
  double step_ms;
} hobak_tuning;
int hobak_batch_get_tuning(hobak_batch b, hobak_tuning* out);
/* Which inner-PCG path each scene takes under the current tuning (no
 * reference counterpart): cluster_ctas[s] = the CTAs of scene s's
 * thread-block cluster, or 0 for the batch-wide tile path. */
int hobak_batch_pcg_path(hobak_batch b, int* cluster_ctas);
/* Per-scene override of that choice (no reference counterpart): ctas = 1, 2,
 * 4, 8 or 16 solves the scene in a cluster of that size when it fits (its
 * vectors in the CTAs' shared memory), -1 keeps it on the tile path, 0 leaves
 * it to the batch's tuning.  Applies from the next step; it depends only on
 * the scene, so a scene given the same override alone and in a batch takes
 * the same path. */
int hobak_batch_set_scene_cluster(hobak_batch b, int scene, int ctas);
int hobak_batch_set_tuning(hobak_batch b, const hobak_tuning* t);
/* Autotuner: times the element kernel per CTA size and the assembly kernel
 * per CTA size (reps launches each, CUDA events), then whole steps for every
 * (PCG path and cluster cap, tile size, chunk) from the batch's current state (restored before
 * every trial and at the end, so the batch's trajectory is unchanged), and
 * applies the fastest shape.  out may be NULL. */
int hobak_batch_autotune(hobak_batch b, int reps, hobak_tuning* out);

/* ---- continuous-batching server (no reference counterpart) ----
 * Scene-timestep jobs admitted FIFO under a device-memory budget into
 * batches ("cohorts", one per admission round) that step on their own
 * streams; hobak_server_pump relaunches each cohort as soon as its own step
 * has completed, hobak_server_tick steps all cohorts in lock step.  Finished
 * jobs are parked and read back; a cohort whose finished jobs hold at least
 * merge_fraction of it, or any cohort with a finished job while jobs are
 * queued, is re-packed with the queued arrivals that fit (built on a host
 * thread when async_build, swapped in at its next step boundary with the
 * running jobs' state carried over), which frees the finished jobs' device
 * memory.  Each job's result is bitwise the same as the job run alone in
 * its own batch with the same solver options and tuning.  One host thread
 * drives a server; its batches use the solver options given here. */
#define HOBAK_JOB_QUEUED 0
#define HOBAK_JOB_RUNNING 1    /* admitted: in a cohort, or in one being built */
#define HOBAK_JOB_FINISHED 2
#define HOBAK_JOB_FAILED 3     /* its cohort could not be built (the round that found it returned the error) */
typedef struct hobak_server_t* hobak_server;
typedef struct hobak_server_opts {
  long long budget_bytes;  /* device memory the server's batches may hold (estimates until built) */
  int max_admit;           /* jobs per new cohort at most (default 64) */
  int max_cohort;          /* jobs per re-packed cohort at most (default 64) */
  int merge;               /* 1: re-pack cohorts (default 1) */
  double merge_fraction;   /* re-pack once this share of a cohort's jobs finished (default 0.5) */
  int async_build;         /* 1: build cohorts on a host thread (default 0) */
  int keep_results;        /* 1: read back every finished job's x, v (default 1) */
  int use_tuning;          /* 1: apply `tuning` to every cohort (default 0: the library's defaults) */
  hobak_tuning tuning;
} hobak_server_opts;
typedef struct hobak_server_stats {
  long long used_bytes;    /* device bytes held or reserved by the server's batches */
  int cohorts, queued, building, merges, merged_arrivals, finished;
  long long ticks;         /* cohort steps completed */
  double now_s;            /* the server's clock (seconds), as in hobak_job_info */
} hobak_server_stats;
typedef struct hobak_job_info {
  int state;               /* HOBAK_JOB_* */
  int done_steps, nsteps, nv;
  double submitted_s, admitted_s, finished_s;  /* server clock; -1 until then */
} hobak_job_info;
void hobak_default_server_opts(hobak_server_opts* opts);
int hobak_server_create(const hobak_server_opts* opts, const hobak_solver_opts* solver, hobak_server* out);
/* Copies the scene; contact = {eps, stiffness, beta} turns vertex-face
 * contact on for this job (NULL: off).  Refuses a job whose estimated
 * footprint exceeds the whole budget. */
int hobak_server_submit(hobak_server s, const hobak_scene_desc* scene, int nsteps, const double* contact, int* job);
/* One scheduling round; *job_steps = job-steps completed in it. */
int hobak_server_pump(hobak_server s, int* job_steps);
int hobak_server_tick(hobak_server s, int* job_steps);
int hobak_server_idle(hobak_server s);  /* 1: nothing queued, building or running */
int hobak_server_get_stats(hobak_server s, hobak_server_stats* out);
/* A job's state; step_ms (done_steps values: each step's latency, launch to
 * completion of its cohort's step), x and v (3 nv each, finished jobs with
 * keep_results) may be NULL. */
int hobak_server_job(hobak_server s, int job, hobak_job_info* info, double* step_ms, double* x, double* v);
int hobak_server_destroy(hobak_server s);

#ifdef __cplusplus
}
#endif
#endif /* HOBAK_GPU_H */
