// timing_wrap.cpp -- TEST INFRASTRUCTURE: timing of the CPU build of the reference,
// linked with -Wl,--wrap on AlgoGas and Transport.
//
// main() calls AlgoGas once per DT (src/Main.cu:332) and AlgoGas calls Transport
// once per hydro substep (src/SourceEuler.cu:293).  These wrappers count the
// substeps and time each AlgoGas call with a monotonic clock, and print one line
// per DT to stderr:
//     REFSTEP <dt index> <substeps in this DT> <seconds in this AlgoGas call>
// so a benchmark reads the reference's own step time without the output dumps.
#include <chrono>
#include <cstdio>

struct force;
struct planetary_system;

extern "C" void __real__Z7AlgoGasP5forcePdS1_S1_S1_S1_P16planetary_systemi(force *, double *, double *, double *,
                                                                            double *, double *, planetary_system *,
                                                                            int);
extern "C" void __real__Z9TransportPdS_S_S_S_d(double *, double *, double *, double *, double *, double);

static long g_substeps = 0;

extern "C" void __wrap__Z9TransportPdS_S_S_S_d(double *a, double *b, double *c, double *d, double *e, double dt) {
  g_substeps++;
  __real__Z9TransportPdS_S_S_S_d(a, b, c, d, e, dt);
}

extern "C" void __wrap__Z7AlgoGasP5forcePdS1_S1_S1_S1_P16planetary_systemi(force *f, double *dens, double *vrad,
                                                                            double *vtheta, double *energy,
                                                                            double *label, planetary_system *sys,
                                                                            int step) {
  const long s0 = g_substeps;
  const auto t0 = std::chrono::steady_clock::now();
  __real__Z7AlgoGasP5forcePdS1_S1_S1_S1_P16planetary_systemi(f, dens, vrad, vtheta, energy, label, sys, step);
  const double sec = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  std::fprintf(stderr, "REFSTEP %d %ld %.9f\n", step, g_substeps - s0, sec);
  std::fflush(stderr);
}
