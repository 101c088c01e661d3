// kapsel_main.cpp -- command-line driver: a kapsel input UDF run on the GPU.
//
//   icep_kapsel -I input.udf [-O out_dir] [-R checkpoint] [--precision fp64|mixed]
//               [--solver ref|spectral] [--steps N]
//
// The counterpart of the reference's main (sp_3d_ns.cxx:367-560) for this
// path: read the input (icep_udf_read), set up the state
// (Init_potential_dielectric and the ion densities for electrolytes, or a
// restart from an icep checkpoint), then GTS * Num_snap steps. Every GTS
// steps one line per particle goes to out_dir/particles_<ts>.dat
// (spec, x, v, omega, q) and a status line to stderr; at the end the state is
// written to out_dir/restart.ckpt (icep_save_checkpoint). With output.AVS
// ON and FileType BINARY or ASCII the reference's AVS field and particle
// frames are written too (Init_output and the main loop's frames,
// output.cxx:15-31, sp_3d_ns.cxx:482-497) into output.ON.Out_dir; EXTENDED
// (HDF5) output is refused, as by a reference built without it. Exit status
// 0 on success, else the library's status code.
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/stat.h>

#include <string>
#include <vector>

#include "../../include/icep_gb300.h"

static int usage() {
  fprintf(stderr,
          "usage: icep_kapsel -I input.udf [-O out_dir] [-R checkpoint] [--precision fp64|mixed]\n"
          "                   [--solver ref|spectral] [--steps N]\n");
  return 2;
}

static int check(icep_ctx *ctx, int st, const char *what) {
  if (st != ICEP_OK) fprintf(stderr, "icep_kapsel: %s failed (%d): %s\n", what, st, ctx ? icep_last_error(ctx) : "");
  return st;
}

static int dump(icep_ctx *ctx, const std::string &dir, int np, std::vector<icep_particle> &buf) {
  int ts = 0;
  double time = 0.0;
  icep_get_time(ctx, &ts, &time);
  int st = icep_get_particles(ctx, buf.data());
  if (st) return check(ctx, st, "get_particles");
  char name[64];
  snprintf(name, sizeof(name), "/particles_%08d.dat", ts);
  FILE *fp = fopen((dir + name).c_str(), "w");
  if (!fp) {
    fprintf(stderr, "icep_kapsel: cannot write %s%s\n", dir.c_str(), name);
    return ICEP_ERR_IO;
  }
  fprintf(fp, "# ts %d time %.17g\n# spec x y z vx vy vz wx wy wz q0 q1 q2 q3\n", ts, time);
  for (int i = 0; i < np; i++) {
    const icep_particle &p = buf[(size_t)i];
    fprintf(fp, "%d %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g %.17g\n", p.spec,
            p.x[0], p.x[1], p.x[2], p.v[0], p.v[1], p.v[2], p.omega[0], p.omega[1], p.omega[2], p.q[0], p.q[1],
            p.q[2], p.q[3]);
  }
  return fclose(fp) == 0 ? ICEP_OK : ICEP_ERR_IO;
}

int main(int argc, char **argv) {
  std::string input, out = ".", restart;
  int precision = -1, solver = -1;
  long steps = -1;
  for (int i = 1; i < argc; i++) {
    const std::string a = argv[i];
    auto next = [&](std::string &v) {
      if (i + 1 >= argc) return false;
      v = argv[++i];
      return true;
    };
    std::string v;
    if (a.rfind("-I", 0) == 0 && a.size() > 2) input = a.substr(2);
    else if (a == "-I") { if (!next(input)) return usage(); }
    else if (a.rfind("-O", 0) == 0 && a.size() > 2) out = a.substr(2);
    else if (a == "-O") { if (!next(out)) return usage(); }
    else if (a == "-R") { if (!next(restart)) return usage(); }
    else if (a == "--precision" && next(v)) precision = (v == "mixed") ? ICEP_MIXED : (v == "fp64") ? ICEP_FP64 : -2;
    else if (a == "--solver" && next(v)) solver = (v == "spectral") ? ICEP_SOLVER_SPECTRAL : (v == "ref") ? ICEP_SOLVER_REF : -2;
    else if (a == "--steps" && next(v)) steps = atol(v.c_str());
    else return usage();
  }
  if (input.empty() || precision == -2 || solver == -2) return usage();
  icep_params p;
  int np = 0, gts = 0, nsnap = 0;
  char err[512];
  int st = icep_udf_read(input.c_str(), &p, nullptr, 0, &np, &gts, &nsnap, err, sizeof(err));
  if (st) {
    fprintf(stderr, "icep_kapsel: %s: %s\n", input.c_str(), err);
    return st;
  }
  std::vector<icep_particle> parts((size_t)(np > 0 ? np : 1));
  st = icep_udf_read(input.c_str(), &p, parts.data(), np, &np, &gts, &nsnap, err, sizeof(err));
  if (st) {
    fprintf(stderr, "icep_kapsel: %s: %s\n", input.c_str(), err);
    return st;
  }
  // output.AVS (input.cxx:1782-1830)
  std::string avs_dir, avs_name;
  int avs_ascii = -1;
  {
    char v[512];
    if (icep_udf_value(input.c_str(), "output.AVS", v, sizeof(v)) == ICEP_OK && std::string(v) == "ON") {
      char d[512], n[512], t[64];
      if (icep_udf_value(input.c_str(), "output.ON.Out_dir", d, sizeof(d)) ||
          icep_udf_value(input.c_str(), "output.ON.Out_name", n, sizeof(n)) ||
          icep_udf_value(input.c_str(), "output.ON.FileType", t, sizeof(t))) {
        fprintf(stderr, "icep_kapsel: %s: output.ON is incomplete\n", input.c_str());
        return ICEP_ERR_ARG;
      }
      const std::string type(t);
      if (type == "EXTENDED") {
        fprintf(stderr, "icep_kapsel: EXTENDED (HDF5) output is not built; use BINARY or ASCII\n");
        return ICEP_ERR_UNSUPPORTED;
      }
      if (p.sw_eq != ICEP_ELECTROLYTE) {
        fprintf(stderr, "icep_kapsel: AVS field output is built for the electrolyte model only\n");
        return ICEP_ERR_UNSUPPORTED;
      }
      avs_dir = d;
      avs_name = n;
      avs_ascii = type == "ASCII" ? 1 : 0;
    }
  }
  if (precision >= 0) p.precision = precision;
  if (solver >= 0) p.solver = solver;
  mkdir(out.c_str(), 0755);
  int cst = 0;
  icep_ctx *ctx = icep_create(&p, parts.data(), np, &cst);
  if (!ctx) {
    fprintf(stderr, "icep_kapsel: icep_create failed (%d)\n", cst);
    return cst ? cst : ICEP_ERR_CUDA;
  }
  if (!restart.empty()) st = check(ctx, icep_load_checkpoint(ctx, restart.c_str()), "load_checkpoint");
  else st = check(ctx, icep_init_state(ctx), "init_state");
  const long total = steps >= 0 ? steps : (long)gts * nsnap;
  fprintf(stderr, "# icep_kapsel: %dx%dx%d, %d particles, dt %.6g, %ld steps (GTS %d)\n", p.nx, p.ny, p.nz, np, p.dt,
          total, gts);
  std::vector<icep_particle> buf((size_t)(np > 0 ? np : 1));
  if (!st && avs_ascii >= 0) {
    st = icep_avs_init(avs_dir.c_str(), avs_name.c_str(), avs_ascii, p.nx, p.ny, p.nz, p.dx, nsnap + 1, np);
    if (st) fprintf(stderr, "icep_kapsel: cannot write the AVS headers in %s\n", avs_dir.c_str());
  }
  // a frame at the start, unless resumed (the reference skips the resumed step's frame)
  if (!st && avs_ascii >= 0 && restart.empty())
    st = check(ctx, icep_output_avs(ctx, avs_dir.c_str(), avs_name.c_str(), avs_ascii), "output_avs");
  if (!st) st = dump(ctx, out, np, buf);
  for (long k = 0; k < total && !st; k++) {
    st = check(ctx, icep_step(ctx, 1), "step");
    if (!st && gts > 0 && (k + 1) % gts == 0) {
      int it = 0;
      double e = 0.0;
      long mv = 0;
      icep_solver_stats(ctx, &it, &e, &mv);
      int ts = 0;
      double t = 0.0;
      icep_get_time(ctx, &ts, &t);
      fprintf(stderr, "# ts %d time %.6g poisson iterations %d residual %.3g\n", ts, t, it, e);
      if (avs_ascii >= 0)
        st = check(ctx, icep_output_avs(ctx, avs_dir.c_str(), avs_name.c_str(), avs_ascii), "output_avs");
      if (!st) st = dump(ctx, out, np, buf);
    }
  }
  if (!st) st = check(ctx, icep_save_checkpoint(ctx, (out + "/restart.ckpt").c_str()), "save_checkpoint");
  icep_destroy(ctx);
  return st;
}
