// params.cpp -- the reference's .par / .cfg parameter interface.
//
// Restates ReadVariables / SearchVariable (src/Interpret.cu:36-212), the defaults
// of include/Param.cuh:51-104 and src/Interpret.cu:22-31, the CLI switches of
// src/Main.cu:115-179 and InitPlanetarySystem (src/Psys.cu:86-217).  Same key
// names, same case folding, same "first token after \t :=>_" value rule, same
// derived flags.  Where the reference calls exit(1) this returns an error code.
#include <cctype>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/fargo_gb300.h"

namespace {

void set_str(char *dst, size_t cap, const char *src) {
  std::snprintf(dst, cap, "%s", src);
}

// Raw values as the reference keeps them (strings compared after the file is read).
struct RawStrings {
  std::string innerboundary = "WALL", labeladvection = "NO", transport = "FAST";
  std::string radialspacing = "ARITHMETIC", disk = "YES", frame = "FIXED";
  std::string outersourcemass = "NO", writedensity = "YES", writevelocity = "YES";
  std::string writeenergy = "NO", writetemperature = "NO", writedivv = "NO", writeqplus = "NO";
  std::string indirectterm = "YES", excludehill = "NO", selfgravity = "NO", cicplanet = "NO";
  std::string forcedcircular = "NO", zmplus = "NO", adiabatic = "NO", cooling = "NO";
};

// SearchVariable src/Interpret.cu:36-96
void search_variable(const char *name, const char *stringval, fargo_params *p, RawStrings &s) {
  double temp = 0.0;
  std::sscanf(stringval, "%lf", &temp);
  auto is = [&](const char *k) { return std::strcmp(name, k) == 0; };
  if (is("DT")) p->dt = temp;
  if (is("SIGMA0")) p->sigma0 = temp;
  if (is("NINTERM")) p->ninterm = (int)temp;
  if (is("NTOT")) p->ntot = (int)temp;
  if (is("OUTPUTDIR")) set_str(p->outputdir, sizeof(p->outputdir), stringval);
  if (is("INNERBOUNDARY")) s.innerboundary = stringval;
  if (is("LABELADVECTION")) s.labeladvection = stringval;
  if (is("TRANSPORT")) s.transport = stringval;
  if (is("PLANETCONFIG")) set_str(p->planetconfig, sizeof(p->planetconfig), stringval);
  if (is("MASSTAPER")) p->masstaper = temp;
  if (is("RADIALSPACING")) s.radialspacing = stringval;
  if (is("NRAD")) p->nrad = (int)temp;
  if (is("NSEC")) p->nsec = (int)temp;
  if (is("RMIN")) p->rmin = temp;
  if (is("RMAX")) p->rmax = temp;
  if (is("THICKNESSSMOOTHING")) p->thicknesssmoothing = temp;
  if (is("ROCHESMOOTHING")) p->rochesmoothing = temp;
  if (is("ASPECTRATIO")) p->aspectratio = temp;
  if (is("VISCOSITY")) p->viscosity = temp;
  if (is("ALPHAVISCOSITY")) p->alphaviscosity = temp;
  if (is("SIGMASLOPE")) p->sigmaslope = temp;
  if (is("RELEASERADIUS")) p->releaseradius = temp;
  if (is("RELEASEDATE")) p->releasedate = temp;
  if (is("OMEGAFRAME")) p->omegaframe = temp;
  if (is("DISK")) s.disk = stringval;
  if (is("FRAME")) s.frame = stringval;
  if (is("OUTERSOURCEMASS")) s.outersourcemass = stringval;
  if (is("WRITEDENSITY")) s.writedensity = stringval;
  if (is("WRITEVELOCITY")) s.writevelocity = stringval;
  if (is("WRITEENERGY")) s.writeenergy = stringval;
  if (is("WRITETEMPERATURE")) s.writetemperature = stringval;
  // src/Interpret.cu:74 assigns the *number* to the string, so the comparison with
  // "YES" at line 147 never succeeds: WriteDivV cannot be enabled from a .par file.
  if (is("WRITEDIVV")) s.writedivv = std::string(1, (char)(int)temp);
  if (is("WRITEQPLUS")) s.writeqplus = stringval;
  if (is("INDIRECTTERM")) s.indirectterm = stringval;
  if (is("EXCLUDEHILL")) s.excludehill = stringval;
  if (is("IMPOSEDDISKDRIFT")) p->imposeddiskdrift = temp;
  if (is("FLARINGINDEX")) p->flaringindex = temp;
  if (is("ECCENTRICITY")) p->eccentricity = temp;
  if (is("CAVITYRADIUS")) p->cavityradius = temp;
  if (is("CAVITYRATIO")) p->cavityratio = temp;
  if (is("CAVITYWIDTH")) p->cavitywidth = temp;
  if (is("TRANSITIONRADIUS")) p->transitionradius = temp;
  if (is("TRANSITIONRATIO")) p->transitionratio = temp;
  if (is("TRANSITIONWIDTH")) p->transitionwidth = temp;
  if (is("LAMBDADOUBLING")) p->lambdadoubling = temp;
  if (is("SELFGRAVITY")) s.selfgravity = stringval;
  if (is("CICPLANET")) s.cicplanet = stringval;
  if (is("FORCEDCIRCULAR")) s.forcedcircular = stringval;
  if (is("ZMPLUS")) s.zmplus = stringval;
  if (is("ADIABATIC")) s.adiabatic = stringval;
  if (is("ADIABATICINDEX")) p->adiabaticindex = temp;
  if (is("COOLING")) s.cooling = stringval;
  if (is("COOLINGTIME0")) p->coolingtime0 = temp;
  // extensions (keys unknown to the reference, which ignores unknown keys)
  if (is("SIGMANOISE")) p->sigma_noise = temp;
  if (is("ENERGYNOISE")) p->energy_noise = temp;
  if (is("NOISESEED")) p->noise_seed = (unsigned long long)std::strtoull(stringval, nullptr, 10);
}

}  // namespace

extern "C" {

void fargo_params_default(fargo_params *p) {
  std::memset(p, 0, sizeof(*p));
  // include/Param.cuh:51-104
  p->dt = 1.0;
  p->sigma0 = 173.0;
  p->ninterm = 10;
  p->ntot = 1501;
  set_str(p->outputdir, sizeof(p->outputdir), "~masset");
  set_str(p->planetconfig, sizeof(p->planetconfig), "Systems/SolarSystem.cfg");
  p->masstaper = 0.0000001;
  p->nrad = 64;
  p->nsec = 64;
  p->rmin = 1.0;
  p->rmax = 1.0;
  p->thicknesssmoothing = 0.0;
  p->rochesmoothing = 0.0;
  p->aspectratio = 0.05;
  p->viscosity = 0.0;
  p->alphaviscosity = 0.0;
  p->sigmaslope = 0.0;
  p->releaseradius = 0.0;
  p->releasedate = 0.0;
  p->omegaframe = 0.0;
  p->imposeddiskdrift = 0.0;
  p->flaringindex = 0.0;
  p->eccentricity = 0.0;
  p->cavityradius = 0.0;
  p->cavityratio = 1.0;
  p->cavitywidth = 1.0;
  p->transitionradius = 0.0;
  p->transitionratio = 1.0;
  p->transitionwidth = 1.0;
  p->lambdadoubling = 0.0;
  p->adiabaticindex = 1.4;
  p->coolingtime0 = 6.28;
  // src/Interpret.cu:25-31
  p->fast_transport = 1;
  p->indirect_term = 1;
  p->is_disk = 1;
  p->write_density = 1;
  p->write_velocity = 1;
  p->log_grid = 0;
  p->scaling_factor = 1.0;
  p->noise_seed = 1;
}

int fargo_params_read(const char *filename, fargo_params *p) {
  FILE *input = std::fopen(filename, "r");
  if (input == nullptr) return FARGO_ERR_IO;
  RawStrings s;
  char nm[300], line[350], stringval[290];
  double temp = 0.0;
  while (std::fgets(line, 349, input) != nullptr) {
    int success = std::sscanf(line, "%299s ", nm);
    if ((nm[0] != '#') && (success == 1)) {  // '#' begins a comment line
      const char *s1 = line + std::strlen(nm);
      const char *v = s1 + std::strspn(s1, "\t :=>_");
      std::sscanf(v, "%lf", &temp);
      stringval[0] = 0;
      std::sscanf(v, "%289s ", stringval);
      for (size_t i = 0; i < std::strlen(nm); i++) nm[i] = (char)std::toupper((unsigned char)nm[i]);
      search_variable(nm, stringval, p, s);
    }
  }
  std::fclose(input);
  // derived flags, src/Interpret.cu:130-206
  if (s.labeladvection == "YES") p->advect_label = 1;
  if (s.outersourcemass == "YES") p->outer_source_mass = 1;
  if (s.transport == "STANDARD") p->fast_transport = 0;
  if (s.innerboundary == "OPEN") p->open_inner = 1;
  if (s.innerboundary == "NONREFLECTING") p->non_reflecting = 1;
  if (s.innerboundary == "EVANESCENT") p->evanescent = 1;
  if (s.radialspacing == "LOGARITHM") p->log_grid = 1;
  if (s.disk == "NO") p->is_disk = 0;
  if (s.frame == "COROTATING") p->corotating = 1;
  if (s.frame == "GUIDING-CENTER") { p->guiding_center = 1; p->corotating = 1; }
  if (s.writevelocity == "NO") p->write_velocity = 0;
  if (s.writedensity == "NO") p->write_density = 0;
  if (s.writeenergy == "YES") p->write_energy = 1;
  if (s.writetemperature == "YES") p->write_temperature = 1;
  if (s.writedivv == "YES") p->write_divv = 1;
  if (s.writeqplus == "YES") p->write_qplus = 1;
  if (s.indirectterm == "NO") p->indirect_term = 0;
  if (s.selfgravity == "YES") p->self_gravity = 1;
  if (s.selfgravity == "Z") { p->self_gravity = 1; p->sg_zero_mode = 1; }
  if (s.adiabatic == "YES") { p->adiabatic = 1; p->write_temperature = 1; }
  if (s.cooling == "YES") p->cooling = 1;
  if (p->adiabatic && p->adiabaticindex == 1.0) p->adiabatic = 0;
  if (s.writeenergy == "NO") p->write_energy = 0;
  if (s.excludehill == "YES") p->exclude_hill = 1;
  if (s.cicplanet == "YES") p->cic_planet = 1;
  if (s.forcedcircular == "YES") p->forced_circular = 1;
  if (p->alphaviscosity != 0.0 && p->viscosity != 0.0) return FARGO_ERR_INVALID;
  if (p->alphaviscosity != 0.0) p->viscosity_alpha = 1;
  if (p->thicknesssmoothing != 0.0 && p->rochesmoothing != 0.0) return FARGO_ERR_INVALID;
  if (p->thicknesssmoothing <= 0.0 && p->rochesmoothing <= 0.0) return FARGO_ERR_INVALID;
  if (p->rochesmoothing != 0.0) p->roche_smoothing = 1;
  // Energy() in src/Theo.cu:234-238 exits on gamma == 1 with an energy equation
  return FARGO_OK;
}

// src/Main.cu:115-151: only the switches that change the computed state are kept;
// the others are accepted and ignored, as the reference ignores most of them.
int fargo_params_apply_switches(const char *sw, fargo_params *p) {
  if (!sw || sw[0] != '-') return FARGO_ERR_INVALID;
  if (std::strspn(sw, "-secndovtpfamzib0123456789") != std::strlen(sw)) return FARGO_ERR_INVALID;
  if (std::strchr(sw, 'c')) p->sloppy_cfl = 1;
  if (std::strchr(sw, 'b')) p->centrifugal_balance = 1;
  return FARGO_OK;
}

// FindNumberOfPlanets + InitPlanetarySystem, src/Psys.cu:86-217
int fargo_planets_read(const char *filename, const fargo_params *p, fargo_planet *out, int cap, int *nb) {
  FILE *input = std::fopen(filename, "r");
  if (input == nullptr) return FARGO_ERR_IO;
  char s[512], nm[512], test1[512], test2[512];
  int count = 0;
  while (std::fgets(s, 510, input) != nullptr) {
    if (!std::isalpha((unsigned char)s[0])) continue;
    std::sscanf(s, "%511s ", nm);
    const char *s1 = s + std::strlen(nm);
    double dist = 0, mass = 0, accret = 0;
    test1[0] = test2[0] = 0;
    std::sscanf(s1 + std::strspn(s1, "\t :=>_"), "%lf %lf %lf %511s %511s", &dist, &mass, &accret, test1, test2);
    if (count < cap) {
      fargo_planet &b = out[count];
      int feeldis = 1, feelothers = 1;
      if (std::tolower((unsigned char)test1[0]) == 'n') feeldis = 0;
      if (std::tolower((unsigned char)test2[0]) == 'n') feelothers = 0;
      b.mass = mass;
      b.x = dist * (1.0 + p->eccentricity);
      b.y = 0.0;
      b.vy = std::sqrt(1.0 * (1.0 + mass) / dist) * std::sqrt((1.0 - p->eccentricity) / (1.0 + p->eccentricity));
      b.vx = -0.0000000001 * b.vy;
      b.acc = accret;
      b.feel_disk = feeldis;
      b.feel_others = feelothers;
    }
    count++;
  }
  std::fclose(input);
  *nb = count;
  return count > cap ? FARGO_ERR_INVALID : FARGO_OK;
}

}  // extern "C"
