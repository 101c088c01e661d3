// avs.cpp -- AVS/Express field and particle output, the reference's default
// writers (avs_output.cxx, avs_output_p.cxx) for the electrolyte model:
// the same file names, header text and float32 payloads, so that tools
// reading the reference's output read these files unchanged.
//
//   <out_dir>/<name>.fld          field header + one description per frame
//   <out_dir>/<name>.cod          uniform-field extents (six %g lines)
//   <out_dir>/avs/<name>_<ts>.dat 7 fields (ux uy uz phi surface_charge rho
//                                 e_potential), float32, x fastest
//   <out_dir>/<name>p.fld         particle header + one description per frame
//   <out_dir>/avs/<name>p_<ts>.cod positions (z, y, x components)
//   <out_dir>/avs/<name>p_<ts>.dat radius and the body axes
// Host code only; the fields come from icep_charge_field_data.
#include <stdio.h>
#include <sys/stat.h>
#include <sys/types.h>

#include <string>
#include <vector>

#include "../../include/icep_gb300.h"

namespace {

const int kVeclen = 7;  // Veclen_charge (avs_output.cxx:13)
const char *kLabel = "ux uy uz phi surface_charge rho e_potential";
const int kVeclenP = 10;  // Veclen_p (avs_output_p.cxx:10)
const char *kLabelP = "Radius x1 x2 x3 y1 y2 y3 z1 z2 z3";

struct Names {  // Set_avs_parameters (avs_output.cxx:146-186)
  std::string fld_file, cod_file, out_cod, out_pfx, pfld_file, out_ppfx, dir;
  Names(const char *out_dir, const char *name) : dir(out_dir) {
    const std::string n(name);
    out_cod = n + ".cod";
    cod_file = dir + "/" + out_cod;
    fld_file = dir + "/" + n + ".fld";
    out_pfx = "avs/" + n + "_";
    pfld_file = dir + "/" + n + "p.fld";
    out_ppfx = "avs/" + n + "p_";
  }
};

bool make_dir(const std::string &d) {
  struct stat st;
  if (stat(d.c_str(), &st) == 0) return S_ISDIR(st.st_mode);
  return mkdir(d.c_str(), 0755) == 0;
}

// closes fp and reports whether everything reached the file
bool close_ok(FILE *fp, bool ok) {
  if (ferror(fp)) ok = false;
  return fclose(fp) == 0 && ok;
}

// rotation matrix of a unit quaternion q = (s, v) (the body axes in the lab
// frame as columns: R[a][b] = e_b . lab axis a)
void rotation(const double *q, double R[3][3]) {
  const double q0 = q[0], q1 = q[1], q2 = q[2], q3 = q[3];
  R[0][0] = 1.0 - 2.0 * (q2 * q2 + q3 * q3);
  R[0][1] = 2.0 * (q1 * q2 - q0 * q3);
  R[0][2] = 2.0 * (q1 * q3 + q0 * q2);
  R[1][0] = 2.0 * (q1 * q2 + q0 * q3);
  R[1][1] = 1.0 - 2.0 * (q1 * q1 + q3 * q3);
  R[1][2] = 2.0 * (q2 * q3 - q0 * q1);
  R[2][0] = 2.0 * (q1 * q3 - q0 * q2);
  R[2][1] = 2.0 * (q2 * q3 + q0 * q1);
  R[2][2] = 1.0 - 2.0 * (q1 * q1 + q2 * q2);
}

}  // namespace

extern "C" {

int icep_avs_init(const char *out_dir, const char *out_name, int ascii, int nx, int ny, int nz, double dx, int nstep,
                  int n_particles) {
  if (!out_dir || !out_name || nx < 1 || ny < 1 || nz < 1 || n_particles < 0) return ICEP_ERR_ARG;
  (void)ascii;  // the headers do not depend on the file type
  const Names nm(out_dir, out_name);
  if (!make_dir(nm.dir) || !make_dir(nm.dir + "/avs")) return ICEP_ERR_IO;
  // Init_avs (avs_output.cxx:46-144), the electrolyte labels, uniform field
  FILE *fp = fopen(nm.fld_file.c_str(), "w");
  if (!fp) return ICEP_ERR_IO;
  fprintf(fp, "# AVS field file\n");
  fprintf(fp, "ndim=%d\n", 3);
  fprintf(fp, "dim1=%d\n", nx);
  fprintf(fp, "dim2=%d\n", ny);
  fprintf(fp, "dim3=%d\n", nz);
  fprintf(fp, "nspace=%d\n", 3);
  fprintf(fp, "veclen=%d\n", kVeclen);
  fprintf(fp, "data=float\n");
  fprintf(fp, "field=uniform\n");
  fprintf(fp, "nstep=%d\n", nstep);
  fprintf(fp, "label = %s\n", kLabel);
  if (!close_ok(fp, true)) return ICEP_ERR_IO;
  fp = fopen(nm.cod_file.c_str(), "wb");
  if (!fp) return ICEP_ERR_IO;
  fprintf(fp, "%g\n%g\n%g\n%g\n%g\n%g\n", (double)0 * dx, (double)(nx - 1) * dx, (double)0 * dx,
          (double)(ny - 1) * dx, (double)0 * dx, (double)(nz - 1) * dx);
  if (!close_ok(fp, true)) return ICEP_ERR_IO;
  if (n_particles > 0) {  // Init_avs_p (avs_output_p.cxx:13-27)
    fp = fopen(nm.pfld_file.c_str(), "w");
    if (!fp) return ICEP_ERR_IO;
    fprintf(fp, "# AVS field file\n");
    fprintf(fp, "ndim=%d\n", 1);
    fprintf(fp, "dim1=%d\n", n_particles);
    fprintf(fp, "nspace=%d\n", 3);
    fprintf(fp, "veclen=%d\n", kVeclenP);
    fprintf(fp, "data=float\n");
    fprintf(fp, "field=irregular\n");
    fprintf(fp, "nstep=%d\n", nstep);
    fprintf(fp, "label = %s\n", kLabelP);
    if (!close_ok(fp, true)) return ICEP_ERR_IO;
  }
  return ICEP_OK;
}

int icep_avs_charge_frame(const char *out_dir, const char *out_name, int ascii, int nx, int ny, int nz, int ts,
                          double time, const double *const *fields) {
  if (!out_dir || !out_name || !fields || nx < 1 || ny < 1 || nz < 1) return ICEP_ERR_ARG;
  for (int v = 0; v < kVeclen; v++)
    if (!fields[v]) return ICEP_ERR_ARG;
  const Names nm(out_dir, out_name);
  // Add_field_description (avs_output.cxx:203-258)
  FILE *fp = fopen(nm.fld_file.c_str(), "a");
  if (!fp) return ICEP_ERR_IO;
  fprintf(fp, "time value = \"step%dtime%g\"\n", ts, time);
  const int data_size = (int)(sizeof(float) * nx * ny * nz);
  for (int n = 0; n < 3; n++)
    fprintf(fp, "coord %d file = %s filetype = ascii skip = %d\n", n + 1, nm.out_cod.c_str(), n * 2);
  for (int n = 0; n < kVeclen; n++) {
    if (!ascii)
      fprintf(fp, "variable %d file = %s%d.dat filetype = binary skip = %d\n", n + 1, nm.out_pfx.c_str(), ts,
              n * data_size);
    else
      fprintf(fp, "variable %d file = %s%d.dat filetype = ascii skip = 2 offset = %d stride = %d\n", n + 1,
              nm.out_pfx.c_str(), ts, n, kVeclen);
  }
  fprintf(fp, "EOT\n");
  if (!close_ok(fp, true)) return ICEP_ERR_IO;
  // Output_avs_charge (avs_output.cxx:332-380): x fastest, then y, then z
  const std::string data = nm.dir + "/" + nm.out_pfx + std::to_string(ts) + ".dat";
  fp = fopen(data.c_str(), "wb");
  if (!fp) return ICEP_ERR_IO;
  const long nz_ = 2 * (nz / 2 + 1);
  bool ok = true;
  if (!ascii) {
    std::vector<float> buf((size_t)nx * ny * nz);
    for (int v = 0; v < kVeclen && ok; v++) {
      size_t q = 0;
      for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
          for (int i = 0; i < nx; i++) buf[q++] = (float)fields[v][((long)i * ny + j) * nz_ + k];
      ok = fwrite(buf.data(), sizeof(float), buf.size(), fp) == buf.size();
    }
  } else {
    fprintf(fp, "timesteps=%d time=%f\n%s\n", ts, time, kLabel);
    for (int k = 0; k < nz; k++)
      for (int j = 0; j < ny; j++)
        for (int i = 0; i < nx; i++) {
          const long im = ((long)i * ny + j) * nz_ + k;
          fprintf(fp, "%.3g %.3g %.3g %.3g %.3g %.3g %.3g\n", fields[0][im], fields[1][im], fields[2][im],
                  fields[3][im], fields[4][im], fields[5][im], fields[6][im]);
        }
  }
  return close_ok(fp, ok) ? ICEP_OK : ICEP_ERR_IO;
}

int icep_avs_particles(const char *out_dir, const char *out_name, int ascii, int ts, double time,
                       const icep_particle *particles, int n_particles, double radius) {
  if (!out_dir || !out_name || n_particles < 0 || (n_particles > 0 && !particles)) return ICEP_ERR_ARG;
  if (n_particles == 0) return ICEP_OK;  // Output_particle_data writes nothing without particles
  const Names nm(out_dir, out_name);
  // Add_pfield_description (avs_output_p.cxx:29-71)
  FILE *fp = fopen(nm.pfld_file.c_str(), "a");
  if (!fp) return ICEP_ERR_IO;
  fprintf(fp, "time value = \"step%dtime%g\"\n", ts, time);
  const int data_size = (int)(sizeof(float) * n_particles);
  for (int n = 0; n < 3; n++) {
    if (!ascii)
      fprintf(fp, "coord %d file = %s%d.cod filetype = binary skip = %d\n", 3 - n, nm.out_ppfx.c_str(), ts,
              n * data_size);
    else
      fprintf(fp, "coord %d file = %s%d.cod filetype = ascii skip = 0 offset = %d stride =%d\n", 3 - n,
              nm.out_ppfx.c_str(), ts, n, 3);
  }
  for (int n = 0; n < kVeclenP; n++) {
    if (!ascii)
      fprintf(fp, "variable %d file = %s%d.dat filetype = binary skip = %d\n", n + 1, nm.out_ppfx.c_str(), ts,
              n * data_size);
    else
      fprintf(fp, "variable %d file = %s%d.dat filetype = ascii skip = 1 offset = %d stride = %d\n", n + 1,
              nm.out_ppfx.c_str(), ts, n, kVeclenP);
  }
  fprintf(fp, "EOT\n");
  if (!close_ok(fp, true)) return ICEP_ERR_IO;
  // Output_avs_p (avs_output_p.cxx:73-157): positions z, y, x
  const std::string base = nm.dir + "/" + nm.out_ppfx + std::to_string(ts);
  fp = fopen((base + ".cod").c_str(), "wb");
  if (!fp) return ICEP_ERR_IO;
  bool ok = true;
  if (!ascii) {
    std::vector<float> buf((size_t)n_particles);
    for (int d = 0; d < 3 && ok; d++) {
      for (int n = 0; n < n_particles; n++) buf[(size_t)n] = (float)particles[n].x[2 - d];
      ok = fwrite(buf.data(), sizeof(float), buf.size(), fp) == buf.size();
    }
  } else {
    for (int n = 0; n < n_particles; n++)
      fprintf(fp, "%.3g %.3g %.3g\n", particles[n].x[2], particles[n].x[1], particles[n].x[0]);
  }
  if (!close_ok(fp, ok)) return ICEP_ERR_IO;
  fp = fopen((base + ".dat").c_str(), "wb");
  if (!fp) return ICEP_ERR_IO;
  std::vector<double> R((size_t)n_particles * 9);
  for (int n = 0; n < n_particles; n++) rotation(particles[n].q, reinterpret_cast<double(*)[3]>(&R[(size_t)n * 9]));
  ok = true;
  if (!ascii) {
    std::vector<float> buf((size_t)n_particles, (float)radius);
    ok = fwrite(buf.data(), sizeof(float), buf.size(), fp) == buf.size();
    for (int d1 = 0; d1 < 3 && ok; d1++)  // body axes e_x, e_y, e_z
      for (int d2 = 0; d2 < 3 && ok; d2++) {
        for (int n = 0; n < n_particles; n++) buf[(size_t)n] = (float)R[(size_t)n * 9 + d2 * 3 + d1];
        ok = fwrite(buf.data(), sizeof(float), buf.size(), fp) == buf.size();
      }
  } else {
    fprintf(fp, "timesteps=%d time=%f\n%s\n", ts, time, kLabelP);
    for (int n = 0; n < n_particles; n++) {
      const double *r = &R[(size_t)n * 9];
      fprintf(fp, "%.3g %.3g %.3g %.3g %.3g %.3g %.3g %.3g %.3g %.3g\n", radius, r[0], r[3], r[6], r[1], r[4],
              r[7], r[2], r[5], r[8]);
    }
  }
  return close_ok(fp, ok) ? ICEP_OK : ICEP_ERR_IO;
}

}  // extern "C"
