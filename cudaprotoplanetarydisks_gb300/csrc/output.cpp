// output.cpp -- the reference's output files (src/Output.cu, src/SourceEuler.cu:148-160).
//
// OUTPUTDIR/<name>/<name><index>.dat: raw FP64, NRAD*NSEC values, ring-major
// (WriteDiskPolar src/Output.cu:150-181); OUTPUTDIR/planet<k>.dat rows
// (WritePlanetFile src/Output.cu:110-131); dims.dat (WriteDim src/Output.cu:19-35);
// used_rad.dat (src/SourceEuler.cu:148-160).
#include <sys/stat.h>
#include <sys/types.h>

#include <cstdio>
#include <cstdlib>
#include <string>
#include <vector>

#include "fargo_internal.h"

int host_write_field(const std::string &outdir, const char *name, int index, const double *data, size_t n) {
  std::string url = outdir + name;
  struct stat st;
  if (stat(url.c_str(), &st) == -1) mkdir(url.c_str(), 0700);
  char fname[1024];
  std::snprintf(fname, sizeof(fname), "%s/%s%d.dat", url.c_str(), name, index);
  FILE *f = std::fopen(fname, "w");
  if (!f) return FARGO_ERR_IO;
  size_t w = std::fwrite(data, sizeof(double), n, f);
  std::fclose(f);
  return w == n ? FARGO_OK : FARGO_ERR_IO;
}

int host_write_planet_row(const std::string &outdir, int k, int index, const fargo_planet &b, double lost_mass,
                          double physical_time, double omega_frame) {
  char fname[1024];
  std::snprintf(fname, sizeof(fname), "%splanet%d.dat", outdir.c_str(), k);
  FILE *f = std::fopen(fname, "a");
  if (!f) return FARGO_ERR_IO;
  // mdcp and exces_mdcp are never updated by the reference (their calls are
  // commented out at src/Main.cu:302, src/SourceEuler.cu:297-298): zero
  std::fprintf(f, "%d\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\t%.18g\n", index, b.x, b.y,
               b.vx, b.vy, b.mass, lost_mass, physical_time, omega_frame, 0.0, 0.0);
  std::fclose(f);
  return FARGO_OK;
}

int host_write_dims(const fargo_params &p, int nb) {
  std::string fn = std::string(p.outputdir) + "dims.dat";
  FILE *f = std::fopen(fn.c_str(), "w");
  if (!f) return FARGO_ERR_IO;
  int ntotterm = p.ninterm > 0 ? p.ntot / p.ninterm : 0;
  std::fprintf(f, "%d\t%d\t\t%d\t%d\t%f\t%d\t%d\t%d\n", 0, 0, 0, 0, p.rmax, ntotterm, p.nrad, p.nsec);
  std::fclose(f);
  // EmptyPlanetSystemFile src/Output.cu:37-58
  for (int k = 0; k < nb; k++) {
    char name[1024];
    std::snprintf(name, sizeof(name), "%splanet%d.dat", p.outputdir, k);
    FILE *g = std::fopen(name, "w");
    if (!g) return FARGO_ERR_IO;
    std::fclose(g);
  }
  return FARGO_OK;
}

int host_write_used_rad(const fargo_params &p, const HostState &h) {
  std::string fn = std::string(p.outputdir) + "used_rad.dat";
  FILE *f = std::fopen(fn.c_str(), "w");
  if (!f) return FARGO_ERR_IO;
  for (int i = 0; i <= p.nrad; i++) std::fprintf(f, "%.18g\n", h.Radii[i]);
  std::fclose(f);
  return FARGO_OK;
}

// ---- restart (FARGO's -s index; the reference parses the switch but never
// restores anything, src/Main.cu:152-160)

int host_read_field(const std::string &outdir, const char *name, int index, double *data, size_t n) {
  char fname[1024];
  std::snprintf(fname, sizeof(fname), "%s%s/%s%d.dat", outdir.c_str(), name, name, index);
  FILE *f = std::fopen(fname, "r");
  if (!f) return FARGO_ERR_IO;
  const size_t r = std::fread(data, sizeof(double), n, f);
  std::fclose(f);
  return r == n ? FARGO_OK : FARGO_ERR_IO;
}

// Row `index` of planet<k>.dat (the layout host_write_planet_row writes)
int host_read_planet_row(const std::string &outdir, int k, int index, fargo_planet &b, double *lost_mass,
                         double *physical_time, double *omega_frame) {
  char fname[1024];
  std::snprintf(fname, sizeof(fname), "%splanet%d.dat", outdir.c_str(), k);
  FILE *f = std::fopen(fname, "r");
  if (!f) return FARGO_ERR_IO;
  char line[2048];
  int rc = FARGO_ERR_IO;
  while (std::fgets(line, sizeof(line), f)) {
    int idx = -1;
    double v[8];
    if (std::sscanf(line, "%d %lf %lf %lf %lf %lf %lf %lf %lf", &idx, &v[0], &v[1], &v[2], &v[3], &v[4], &v[5], &v[6],
                    &v[7]) == 9 &&
        idx == index) {
      b.x = v[0];
      b.y = v[1];
      b.vx = v[2];
      b.vy = v[3];
      b.mass = v[4];
      *lost_mass = v[5];
      *physical_time = v[6];
      *omega_frame = v[7];
      rc = FARGO_OK;
    }
  }
  std::fclose(f);
  return rc;
}

// Keeps the rows of planet<k>.dat whose index is below `index`
int host_truncate_planet_file(const std::string &outdir, int k, int index) {
  char fname[1024];
  std::snprintf(fname, sizeof(fname), "%splanet%d.dat", outdir.c_str(), k);
  FILE *f = std::fopen(fname, "r");
  if (!f) return FARGO_ERR_IO;
  std::vector<std::string> keep;
  char line[2048];
  while (std::fgets(line, sizeof(line), f))
    if (std::atoi(line) < index) keep.push_back(line);
  std::fclose(f);
  f = std::fopen(fname, "w");
  if (!f) return FARGO_ERR_IO;
  for (const std::string &l : keep) std::fputs(l.c_str(), f);
  std::fclose(f);
  return FARGO_OK;
}

// One row "index\tv0\tv1..." (%.18g) appended to OUTPUTDIR/<file>
int host_append_row(const std::string &outdir, const std::string &file, int index, const double *v, int nv) {
  const std::string fname = outdir + file;
  FILE *f = std::fopen(fname.c_str(), "a");
  if (!f) return FARGO_ERR_IO;
  std::fprintf(f, "%d", index);
  for (int q = 0; q < nv; q++) std::fprintf(f, "\t%.18g", v[q]);
  std::fprintf(f, "\n");
  std::fclose(f);
  return FARGO_OK;
}
