// sg_wrap.cpp -- TEST INFRASTRUCTURE: lets the CPU build of the reference start a
// self-gravitating run, linked with -Wl,--wrap on Init_planetarysys_withSG.
//
// The reference cannot start one: main() calls Init_planetarysys_withSG
// (src/Main.cu:289) before InitEuler allocates SoundSpeed_d, and the function's
// Make1Dprofile(1) (src/SgMain.cu:169, src/Kernels.cu:628-632) copies from that
// null pointer; gpuErrchk exits ("invalid argument", src/Kernels.cu:631).  This
// wrapper replaces only that step.  It gives the planets the circular-orbit speed
// correction of src/SgMain.cu:171-193 with the radial self-gravity acceleration
// averaged in azimuth -- what the comment at src/SgMain.cu:175-177 says the
// profile is -- summed in j order over SG_Accr_d, which compute_selfgravity
// (src/Main.cu:283) has just filled.  The oracle's Init_planetarysys_withSG does
// the same, so the planets' initial speeds agree by construction; everything after
// it (every compute_selfgravity call, the SG velocity kicks, the SG sub-Keplerian
// boundary, the hydro) is the reference's own code.
#include <cmath>

#include "Types.cuh"  // the reference's PlanetarySystem (include/Types.cuh:2-15)

extern int NRAD, NSEC;
extern double *SG_Accr_d, *GLOBAL_AxiSGAccr, *Rmed;
extern double ECCENTRICITY;

extern "C" void __real__Z24Init_planetarysys_withSGP16planetary_system(PlanetarySystem *sys);

extern "C" void __wrap__Z24Init_planetarysys_withSGP16planetary_system(PlanetarySystem *sys) {
  for (int i = 0; i < NRAD; i++) {
    double sum = 0.0;
    for (int j = 0; j < NSEC; j++) sum += SG_Accr_d[(size_t)i * NSEC + j];
    GLOBAL_AxiSGAccr[i] = sum / (double)NSEC;
  }
  for (int k = 0; k < sys->nb; k++) {
    double r = sys->x[k];
    double dist = (double)(r / (1. + ECCENTRICITY));
    int ipl = 0;
    while (Rmed[ipl] <= dist) ipl++;
    double ri = Rmed[ipl];
    double rip1 = Rmed[ipl + 1];
    double dr = rip1 - ri;
    double sgacc = (dist - ri) * GLOBAL_AxiSGAccr[ipl + 1] + (rip1 - dist) * GLOBAL_AxiSGAccr[ipl];
    sgacc /= dr;
    sys->vy[k] *= (double)std::sqrt(1. - dist * dist * sgacc);
  }
}
