// dg_cli.cpp -- `dgcuda`, the command line of the reference's run_dgcuda
// (src/2d/conservation/main.cu:481-974) on top of the C ABI in dg.h.
//
//   dgcuda [OPTIONS] MESH        (.pmsh, or a Gmsh 2.x .msh converted on the fly)
//     -n p        order of the polynomial approximation (0..5)
//     -t steps    number of time steps
//     -T time     end time
//     -v          verbose (time and dt of every step)
//     -c tol      run until max |c_new - c_old| < tol
//     -V every    write output/video/U<var>-<k>.pos every `every` steps
//     -e          evaluate the L2 error against the exact solution
//     -b          benchmark (print the run time)
//     -h          usage
//   options that the reference selects at compile time:
//     --eq advection|euler|shallowwater|maxwell   (equation module)
//     --problem NAME   (adv_sine, adv_linear, euler_vortex, euler_riemann4,
//                       euler_supersonic, sw_hump, sw_test, maxwell_plane,
//                       euler_cylinder, euler_lshock, euler_doublemach,
//                       euler_airfoil, adv_squarehill, adv_rotatinghill,
//                       adv_spin, maxwell_cmirror, maxwell_wscatter, euler_pulse)
//     --reference-settings   start from the problem file's own settings
//                      (limiter, time integrator, Mach, velocity); the
//                      options below override them
//     --scheme rk4|rk2|ssprk3   (time_integrator; default rk4)
//     --limiter        (limiter = LIMITER)
//     --cfl x          (default: 0.5 for rk4, 0.7 for rk2, 0.3 for ssprk3)
//     --gamma g  --gravity g  --velocity ax,ay  --mu m  --eps e
//     --prm a,b,...    problem parameters
//     --field gxx,gxy,gyx,gyy  advection velocity (ax, ay) + grad (x, y)
//     --series t0,a1,w1,f1,a2,w2,f2,...  euler_pulse inflow pressure
//                      1 + sum a_k cos(w_k (t + t0) + f_k)
//     -o DIR           output directory (default "output")
//     --restart FILE   start from a checkpoint (state, bed and time)
//     --checkpoint FILE  write a checkpoint at the end
// Like the reference it writes the final vertex values of U0 to
// DIR/U0-final.pos (write_U, main.cu:69-116) and, with -e, prints
// "L2 U<n> error     = %e".
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "dg.h"

namespace {

void usage() {
  std::printf(
      "\nUsage: dgcuda [OPTIONS] [MESH]\n"
      " Options: [-n] Order of polynomial approximation.\n"
      "          [-t] Number of timesteps.\n"
      "          [-T] End time.\n"
      "          [-v] Verbose.\n"
      "          [-c] Run to convergence of tolerance TOL\n"
      "          [-V] Print out every N timesteps.\n"
      "          [-e] Evaluate the error. Requires an exact solution.\n"
      "          [-b] Benchmark.\n"
      "          [-h] Display this message.\n"
      "          [--eq advection|euler|shallowwater|maxwell] [--problem NAME]\n"
      "          [--scheme rk4|rk2|ssprk3] [--limiter] [--cfl X] [--gamma G]\n"
      "          [--gravity G] [--velocity AX,AY] [--mu M] [--eps E] [--prm A,B,..]\n"
      "          [--reference-settings] [--field GXX,GXY,GYX,GYY]\n"
      "          [--series T0,A1,W1,F1,..] [-o DIR] [--restart FILE] [--checkpoint FILE]\n");
}

std::vector<double> parse_list(const char *s) {
  std::vector<double> v;
  const char *p = s;
  while (*p) {
    char *end;
    double x = std::strtod(p, &end);
    if (end == p) break;
    v.push_back(x);
    p = end;
    if (*p == ',') p++;
  }
  return v;
}

int fail(const char *what) {
  std::fprintf(stderr, "ERROR: %s: %s\n", what, dg_last_error());
  return 1;
}

bool write_pos(dg_solver *s, const std::vector<double> &V, int K, int var,
               const std::string &path) {
  std::vector<double> uv((size_t)3 * K);
  if (dg_eval_vertices(s, var, uv.data()) != DG_OK) return false;
  FILE *f = std::fopen(path.c_str(), "w");
  if (!f) return false;
  std::fprintf(f, "View \"U%i \" {\n", var);
  for (int i = 0; i < K; i++)
    std::fprintf(f,
                 "ST (%.015lf,%.015lf,0,%.015lf,%.015lf,0,%.015lf,%.015lf,0) "
                 "{%.015lf,%.015lf,%.015lf};\n",
                 V[i], V[K + i], V[2 * K + i], V[3 * K + i], V[4 * K + i], V[5 * K + i],
                 uv[i], uv[K + i], uv[2 * K + i]);
  std::fprintf(f, "};");
  std::fclose(f);
  return true;
}

}  // namespace

int main(int argc, char **argv) {
  int p = 1, total_timesteps = -1, verbose = 0, video = 0, convergence = 0, eval_error = 0;
  int benchmark = 0, limiter = 0;
  double endtime = -1, tol = 0, cfl = -1;
  std::string eq_name = "euler", problem = "none", scheme_name = "rk4", outdir = "output";
  std::string restart, checkpoint;
  std::vector<double> field, series;
  const char *pbs[] = {"none", "adv_sine", "adv_linear", "euler_vortex", "euler_riemann4",
                       "euler_supersonic", "sw_hump", "sw_test", "maxwell_plane",
                       "euler_cylinder", "euler_lshock", "euler_doublemach", "euler_airfoil",
                       "adv_squarehill", "adv_rotatinghill", "adv_spin", "maxwell_cmirror",
                       "maxwell_wscatter", "euler_pulse"};
  const int npbs = (int)(sizeof pbs / sizeof pbs[0]);
  dg_params prm;
  dg_params_default(&prm);
  if (argc < 2) {
    usage();
    return 1;
  }
  // the problem's own settings first, so that the options override them
  for (int i = 1; i < argc - 1; i++)
    if (!std::strcmp(argv[i], "--reference-settings")) {
      int pb = -1, sc = DG_RK4;
      for (int j = 1; j + 1 < argc - 1; j++)
        if (!std::strcmp(argv[j], "--problem"))
          for (int k = 0; k < npbs; k++)
            if (!std::strcmp(argv[j + 1], pbs[k])) pb = k;
      if (pb < 0 || dg_params_for_problem(&prm, pb, &sc) != DG_OK) { usage(); return 1; }
      limiter = prm.limiter;
      scheme_name = sc == DG_RK2 ? "rk2" : "rk4";
    }
  for (int i = 1; i < argc; i++)
    if (!std::strcmp(argv[i], "-h")) {
      usage();
      return 1;
    }
  for (int i = 1; i < argc - 1; i++) {
    std::string a = argv[i];
    auto next = [&]() -> const char * {
      if (i + 1 >= argc - 1) {
        usage();
        std::exit(1);
      }
      return argv[++i];
    };
    if (a == "-n") {
      p = std::atoi(next());
      if (p < 0 || p > 5) { usage(); return 1; }
    } else if (a == "-t") {
      total_timesteps = std::atoi(next());
      if (total_timesteps < 0) { usage(); return 1; }
    } else if (a == "-T") {
      endtime = std::atof(next());
      if (endtime < 0) { usage(); return 1; }
    } else if (a == "-V") {
      video = std::atoi(next());
    } else if (a == "-c") {
      convergence = 1;
      tol = std::atof(next());
    } else if (a == "-b") benchmark = 1;
    else if (a == "-e") eval_error = 1;
    else if (a == "-v") verbose = 1;
    else if (a == "-h") { usage(); return 1; }
    else if (a == "--eq") eq_name = next();
    else if (a == "--problem") problem = next();
    else if (a == "--scheme") scheme_name = next();
    else if (a == "--limiter") limiter = 1;
    else if (a == "--reference-settings") continue;
    else if (a == "--field") {
      field = parse_list(next());
      if (field.size() != 4) { usage(); return 1; }
    } else if (a == "--series") {
      series = parse_list(next());
      if (series.size() % 3 != 1 || series.size() > 49) { usage(); return 1; }
    }
    else if (a == "--cfl") cfl = std::atof(next());
    else if (a == "--gamma") prm.gamma = std::atof(next());
    else if (a == "--gravity") prm.gravity = std::atof(next());
    else if (a == "--mu") prm.mu = std::atof(next());
    else if (a == "--eps") prm.eps = std::atof(next());
    else if (a == "--velocity") {
      auto v = parse_list(next());
      if (v.size() != 2) { usage(); return 1; }
      prm.ax = v[0];
      prm.ay = v[1];
    } else if (a == "--prm") {
      auto v = parse_list(next());
      for (size_t k = 0; k < v.size() && k < 8; k++) prm.prm[k] = v[k];
    } else if (a == "-o") outdir = next();
    else if (a == "--restart") restart = next();
    else if (a == "--checkpoint") checkpoint = next();
    else {
      std::fprintf(stderr, "unknown option %s\n", a.c_str());
      usage();
      return 1;
    }
  }
  const char *mesh_path = argv[argc - 1];
  dg_equation eq;
  if (eq_name == "advection") eq = DG_ADVECTION;
  else if (eq_name == "euler") eq = DG_EULER;
  else if (eq_name == "shallowwater") eq = DG_SHALLOW_WATER;
  else if (eq_name == "maxwell") eq = DG_MAXWELL;
  else { usage(); return 1; }
  prm.problem = -1;
  for (int k = 0; k < npbs; k++)
    if (problem == pbs[k]) prm.problem = k;
  if (prm.problem < 0) { usage(); return 1; }
  dg_scheme scheme;
  if (scheme_name == "rk4") scheme = DG_RK4;
  else if (scheme_name == "rk2") scheme = DG_RK2;
  else if (scheme_name == "ssprk3") scheme = DG_SSP_RK3;
  else { usage(); return 1; }
  prm.cfl = cfl > 0 ? cfl : (scheme == DG_RK4 ? 0.5 : scheme == DG_RK2 ? 0.7 : 0.3);
  prm.limiter = limiter;

  dg_mesh *mesh = nullptr;
  const size_t plen = std::strlen(mesh_path);
  const bool gmsh = plen > 4 && !std::strcmp(mesh_path + plen - 4, ".msh");
  if ((gmsh ? dg_mesh_read_gmsh(mesh_path, &mesh) : dg_mesh_read_pmsh(mesh_path, &mesh)) != DG_OK)
    return fail("reading the mesh");
  int K = 0, S = 0;
  dg_mesh_sizes(mesh, &K, &S);
  std::vector<double> V((size_t)6 * K);
  dg_mesh_get_arrays(mesh, V.data(), nullptr, nullptr, nullptr);
  dg_solver *s = nullptr;
  if (dg_solver_create(mesh, eq, p, &prm, 0, &s) != DG_OK) return fail("creating the solver");
  if (!field.empty() && dg_set_velocity_field(s, prm.ax, prm.ay, field.data()) != DG_OK)
    return fail("the velocity field");
  if (!series.empty()) {
    const int n = (int)(series.size() - 1) / 3;
    std::vector<double> amp(n), omega(n), phase(n);
    for (int k = 0; k < n; k++) {
      amp[k] = series[1 + 3 * k];
      omega[k] = series[2 + 3 * k];
      phase[k] = series[3 + 3 * k];
    }
    if (dg_set_inflow_series(s, n, amp.data(), omega.data(), phase.data(), series[0]) != DG_OK)
      return fail("the inflow series");
  }
  if (dg_init(s) != DG_OK) return fail("initial conditions");
  int N = 0, np = 0;
  dg_solver_sizes(s, &N, &np, nullptr, nullptr);
  double dt0 = 0, lam = 0, dmin = 0;
  dg_cfl(s, &dt0, &lam, &dmin);
  std::printf(" ? %i degree polynomial interpolation (local_n_p = %i)\n", p, np);
  std::printf(" ? %i elements\n ? %i sides\n ? min radius = %.015lf\n", K, S, dmin);
  if (endtime == -1 && !convergence) std::printf(" ? total_timesteps = %i\n", total_timesteps);
  else if (endtime != -1 && !convergence) std::printf(" ? endtime = %lf\n", endtime);
  else std::printf(" ? convergence = %lf\n", tol);
  mkdir(outdir.c_str(), 0755);
  if (video > 0) mkdir((outdir + "/video").c_str(), 0755);

  double t = 0.0;
  if (!restart.empty() && dg_load_checkpoint(s, restart.c_str(), &t) != DG_OK)
    return fail("reading the checkpoint");
  auto start = std::chrono::steady_clock::now();
  int steps = 0, vid = 0;
  const bool per_step = verbose || video > 0 || convergence;
  if (!per_step) {
    dg_status st = DG_OK;
    if (endtime >= 0) st = dg_advance_to(s, endtime, scheme, &t, &steps);
    if (st == DG_OK && total_timesteps > 0) {
      st = dg_step(s, total_timesteps, scheme, 0.0, &t);
      steps += total_timesteps;
    }
    if (st != DG_OK) return fail("time integration");
  } else {
    std::vector<double> prev, cur;
    if (convergence) {
      prev.resize((size_t)N * np * K);
      dg_get_state(s, prev.data());
      cur.resize(prev.size());
    }
    if (video > 0) write_pos(s, V, K, 0, outdir + "/video/U0-0.pos"), vid++;
    double conv = 1.0;
    while ((endtime >= 0 && t < endtime) || (total_timesteps > 0 && steps < total_timesteps) ||
           (convergence && conv > tol)) {
      double t0 = t;
      dg_status st;
      if (endtime >= 0 && t < endtime) {
        int n1 = 0;
        dg_cfl(s, &dt0, &lam, &dmin);
        st = t + dt0 > endtime ? dg_advance_to(s, endtime, scheme, &t, &n1)
                               : dg_step(s, 1, scheme, 0.0, &t);
      } else {
        st = dg_step(s, 1, scheme, 0.0, &t);
      }
      if (st != DG_OK) return fail("time integration");
      steps++;
      if (verbose) std::printf("(%i) t = %lf, dt = %lf, max_l = %lf\n", steps, t, t - t0, lam);
      if (convergence) {
        dg_get_state(s, cur.data());
        conv = 0;
        for (size_t k = 0; k < cur.size(); k++) conv = std::fmax(conv, std::fabs(cur[k] - prev[k]));
        prev.swap(cur);
        if (!verbose) std::printf("\r(%i) t = %lf, convergence = %.015lf", steps, t, conv);
      }
      if (video > 0 && steps % video == 0)
        write_pos(s, V, K, 0, outdir + "/video/U0-" + std::to_string(vid++) + ".pos");
    }
    std::printf("\n");
  }
  if (benchmark) {
    double el = std::chrono::duration<double>(std::chrono::steady_clock::now() - start).count();
    std::printf("Runtime: %lf seconds\n", el);
  }
  if (eval_error) {
    std::vector<double> err(N);
    if (dg_l2_error(s, t, err.data()) != DG_OK) return fail("L2 error");
    for (int n = 0; n < N; n++) std::printf("L2 U%i error     = %e\n", n, err[n]);
  }
  if (!write_pos(s, V, K, 0, outdir + "/U0-final.pos")) return fail("writing output");
  if (!checkpoint.empty() && dg_save_checkpoint(s, checkpoint.c_str(), t) != DG_OK)
    return fail("writing the checkpoint");
  std::printf("t = %.15g after %d steps\n", t, steps);
  dg_solver_destroy(s);
  dg_mesh_destroy(mesh);
  return 0;
}
