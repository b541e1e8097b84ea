// A C++ host serving scene-timestep jobs with the library's server
// (hobak_server_*): the jobs arrive in two waves, the server is pumped until
// idle, and every job's final state is written out beside the same scene
// run alone in its own batch, for the caller to compare.
//
// usage: serve_example <in.bin> <out.bin>
//   in:  int32 njobs, then per job: int32 nv, nt, npinned, nsteps, kind;
//        float64 mu, lambda, density, dt, gravity[3]; float64 rest[3 nv];
//        int32 tets[4 nt]; int32 pinned[npinned]; float64 x0[3 nv]
//   out: per job: float64 x[3 nv], v[3 nv] (served), x[3 nv], v[3 nv] (alone)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "hobak_gpu.h"

namespace {

struct Scene {
  int nv = 0, nt = 0, npinned = 0, nsteps = 0, kind = 0;
  double mu = 0, lambda = 0, density = 0, dt = 0, gravity[3] = {0, 0, 0};
  std::vector<double> rest, x0;
  std::vector<int> tets, pinned;
  hobak_scene_desc desc() const {
    hobak_scene_desc d{};
    d.nv = nv;
    d.nt = nt;
    d.rest = rest.data();
    d.tets = tets.data();
    d.material.kind = kind;
    d.material.mu = mu;
    d.material.lambda = lambda;
    d.density = density;
    for (int i = 0; i < 3; i++) d.gravity[i] = gravity[i];
    d.dt = dt;
    d.npinned = npinned;
    d.pinned = pinned.empty() ? nullptr : pinned.data();
    d.x0 = x0.data();
    d.v0 = nullptr;
    return d;
  }
};

template <typename T>
void read(FILE* f, T* p, size_t n) {
  if (fread(p, sizeof(T), n, f) != n) {
    std::fprintf(stderr, "short input\n");
    std::exit(2);
  }
}

void check(int rc, const char* what) {
  if (rc < 0) {
    std::fprintf(stderr, "%s: %s\n", what, hobak_last_error());
    std::exit(1);
  }
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 3) return 2;
  FILE* in = std::fopen(argv[1], "rb");
  if (!in) return 2;
  int njobs = 0;
  read(in, &njobs, 1);
  std::vector<Scene> sc(njobs);
  for (Scene& s : sc) {
    int hdr[5];
    read(in, hdr, 5);
    s.nv = hdr[0], s.nt = hdr[1], s.npinned = hdr[2], s.nsteps = hdr[3], s.kind = hdr[4];
    double par[7];
    read(in, par, 7);
    s.mu = par[0], s.lambda = par[1], s.density = par[2], s.dt = par[3];
    for (int i = 0; i < 3; i++) s.gravity[i] = par[4 + i];
    s.rest.resize(3 * (size_t)s.nv);
    s.tets.resize(4 * (size_t)s.nt);
    s.pinned.resize(s.npinned);
    s.x0.resize(3 * (size_t)s.nv);
    read(in, s.rest.data(), s.rest.size());
    read(in, s.tets.data(), s.tets.size());
    if (s.npinned) read(in, s.pinned.data(), s.pinned.size());
    read(in, s.x0.data(), s.x0.size());
  }
  std::fclose(in);

  hobak_solver_opts opts;
  hobak_default_solver_opts(&opts);
  opts.precision = HOBAK_PRECISION_MIXED;
  hobak_server_opts so;
  hobak_default_server_opts(&so);
  so.budget_bytes = 16LL << 30;
  so.max_admit = 2;  // small cohorts, so later arrivals merge into running ones
  hobak_server srv;
  check(hobak_server_create(&so, &opts, &srv), "hobak_server_create");
  std::vector<int> id(njobs);
  // first wave: two jobs, a few rounds, then the rest while those run
  const int first = njobs < 2 ? njobs : 2;
  for (int k = 0; k < first; k++) {
    hobak_scene_desc d = sc[k].desc();
    check(hobak_server_submit(srv, &d, sc[k].nsteps, nullptr, &id[k]), "hobak_server_submit");
  }
  int steps = 0;
  for (int r = 0; r < 3; r++) check(hobak_server_pump(srv, &steps), "hobak_server_pump");
  for (int k = first; k < njobs; k++) {
    hobak_scene_desc d = sc[k].desc();
    check(hobak_server_submit(srv, &d, sc[k].nsteps, nullptr, &id[k]), "hobak_server_submit");
    check(hobak_server_pump(srv, &steps), "hobak_server_pump");
  }
  while (!hobak_server_idle(srv)) check(hobak_server_pump(srv, &steps), "hobak_server_pump");

  FILE* out = std::fopen(argv[2], "wb");
  if (!out) return 2;
  for (int k = 0; k < njobs; k++) {
    const size_t n = 3 * (size_t)sc[k].nv;
    std::vector<double> x(n), v(n);
    hobak_job_info info;
    check(hobak_server_job(srv, id[k], &info, nullptr, x.data(), v.data()), "hobak_server_job");
    if (info.state != HOBAK_JOB_FINISHED || info.done_steps != sc[k].nsteps) return 3;
    std::fwrite(x.data(), sizeof(double), n, out);
    std::fwrite(v.data(), sizeof(double), n, out);
    // the same scene alone in its own batch
    hobak_scene_desc d = sc[k].desc();
    hobak_batch b;
    check(hobak_batch_create(&d, 1, &opts, &b), "hobak_batch_create");
    check(hobak_batch_step(b, sc[k].nsteps, nullptr), "hobak_batch_step");
    check(hobak_batch_get_state(b, 0, x.data(), v.data()), "hobak_batch_get_state");
    hobak_batch_destroy(b);
    std::fwrite(x.data(), sizeof(double), n, out);
    std::fwrite(v.data(), sizeof(double), n, out);
  }
  std::fclose(out);
  hobak_server_stats st;
  check(hobak_server_get_stats(srv, &st), "hobak_server_get_stats");
  std::printf("jobs %d merges %d merged arrivals %d ticks %lld\n", njobs, st.merges, st.merged_arrivals, st.ticks);
  hobak_server_destroy(srv);
  return 0;
}
