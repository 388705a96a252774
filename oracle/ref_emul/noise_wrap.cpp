// noise_wrap.cpp -- TEST INFRASTRUCTURE: seeded initial noise for the CPU build of the
// reference, linked with -Wl,--wrap on InitGasDensity / InitGasEnergy (called from
// src/Main.cu:258,264).  Same generator and order as the library's SigmaNoise /
// EnergyNoise extension: splitmix64 from FARGO_REF_NOISE_SEED, one draw per cell,
// ring-major, density then energy; Sigma *= 1 + amp * (2u - 1).
#include <cstdint>
#include <cstdlib>

extern int NRAD, NSEC;
// the linker maps the reference's calls of the (mangled) C++ functions to the
// __wrap_ symbols below and __real_ back to the originals
extern "C" void __real__Z14InitGasDensityPd(double *Dens);
extern "C" void __real__Z13InitGasEnergyPd(double *Energy);

static uint64_t g_state;
static bool g_seeded = false;

static uint64_t splitmix64() {
  uint64_t z = (g_state += 0x9E3779B97F4A7C15ULL);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
  return z ^ (z >> 31);
}
static void seed() {
  if (g_seeded) return;
  const char *s = std::getenv("FARGO_REF_NOISE_SEED");
  g_state = s ? std::strtoull(s, nullptr, 10) : 1ULL;
  g_seeded = true;
}
static void apply(double *f, const char *env) {
  const char *a = std::getenv(env);
  const double amp = a ? std::atof(a) : 0.0;
  if (amp == 0.0) return;
  seed();
  for (int i = 0; i < NRAD; i++)
    for (int j = 0; j < NSEC; j++) {
      double u = (double)(splitmix64() >> 11) * (1.0 / 9007199254740992.0);
      f[j + (size_t)i * NSEC] *= 1.0 + amp * (2.0 * u - 1.0);
    }
}

extern "C" void __wrap__Z14InitGasDensityPd(double *Dens) {
  __real__Z14InitGasDensityPd(Dens);
  apply(Dens, "FARGO_REF_SIGMA_NOISE");
}
extern "C" void __wrap__Z13InitGasEnergyPd(double *Energy) {
  __real__Z13InitGasEnergyPd(Energy);
  apply(Energy, "FARGO_REF_ENERGY_NOISE");
}
