// driver.cpp -- fargo_gb300, the command-line driver (the reference's main(),
// src/Main.cu:89-363) on top of the C-ABI.
//
//   echo 0 | fargo_gb300 [-switches] [-s index] [--fp32] [--torques] parameters.par
//
// Reads the device ordinal from standard input like the reference
// (src/Main.cu:92-97; 0 when nothing is given), parses the .par file and the
// planet .cfg (ReadVariables, InitPlanetarySystem), writes dims.dat /
// used_rad.dat / planet<k>.dat, then runs NTOT+1 DT steps, writing the field
// dumps before each step whose index is a multiple of NINTERM
// (src/Main.cu:309-333), and prints the elapsed seconds of the loop.  -s index
// restarts from output `index` of an earlier run in the same OUTPUTDIR (FARGO's
// restart, which the reference parses but never performs): the loop resumes at
// DT step index * NINTERM.  --torques writes the torque logs every DT (UpdateLog,
// whose call the reference keeps commented out at src/Main.cu:315), with the
// reference's TimeStep: the index of the last output written.
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "fargo_gb300.h"

static void usage(const char *exe) {
  std::printf("Usage : %s [-abcdeimnptvz] [-s index] [--fp32] [--torques] parameters file\n", exe);
  std::exit(1);
}

int main(int argc, char **argv) {
  int device = 0;
  std::printf("enter gpu device: ");
  if (std::scanf("%d", &device) != 1) device = 0;
  std::printf("\n");
  if (cudaSetDevice(device) != cudaSuccess) {
    std::fprintf(stderr, "cannot select device %d\n", device);
    return 1;
  }
  if (argc == 1) usage(argv[0]);
  fargo_params p;
  fargo_params_default(&p);
  std::string parfile, switches;
  int precision = FARGO_FP64;
  bool disable = false;
  int restart = -1;
  bool torques = false;
  for (int i = 1; i < argc; i++) {
    if (std::strcmp(argv[i], "--fp32") == 0) {
      precision = FARGO_FP32_BULK;
    } else if (std::strcmp(argv[i], "--torques") == 0) {
      torques = true;
    } else if (argv[i][0] == '-') {
      switches += argv[i] + 1;
      if (std::strchr(argv[i], 'n')) disable = true;
      const bool has_s = std::strchr(argv[i], 's') != nullptr;
      if (has_s || std::strchr(argv[i], 'o') || std::strchr(argv[i], 'f')) i++;  // option value
      if (has_s) {
        restart = i < argc ? std::atoi(argv[i]) : -1;
        if (restart < 0) {
          std::printf("Incorrect restart number\n");
          usage(argv[0]);
        }
      }
    } else {
      parfile = argv[i];
    }
  }
  if (parfile.empty()) usage(argv[0]);
  int rc = fargo_params_read(parfile.c_str(), &p);
  if (rc == FARGO_ERR_IO) {
    std::printf("Unable to read %s . Program stopped. \n", parfile.c_str());
    return 1;
  }
  if (rc != FARGO_OK) {
    std::printf("Inconsistent parameters in %s. Program stopped.\n", parfile.c_str());
    return 1;
  }
  if (!switches.empty() && fargo_params_apply_switches(("-" + switches).c_str(), &p) != FARGO_OK) usage(argv[0]);
  if (disable) return 0;
  fargo_planet planets[64];
  int nb = 0;
  rc = fargo_planets_read(p.planetconfig, &p, planets, 64, &nb);
  if (rc != FARGO_OK) {
    std::fprintf(stderr, "Error : can't find '%s'.\n", p.planetconfig);
    return 1;
  }
  std::printf("%d planet(s) found.\n", nb);
  fargo_ctx *ctx = nullptr;
  rc = fargo_ctx_create(&p, planets, nb, precision, nullptr, &ctx);
  if (rc != FARGO_OK) {
    std::fprintf(stderr, "initialisation failed (status %d)\n", rc);
    return 1;
  }
  // a restart keeps dims.dat and the planet files of the earlier run
  rc = restart >= 0 ? fargo_restart(ctx, restart) : fargo_write_dims(ctx);
  if (rc != FARGO_OK) {
    std::fprintf(stderr, "%s\n", fargo_last_error(ctx));
    fargo_ctx_destroy(ctx);
    return 1;
  }
  if (restart >= 0) std::printf("restarting from output %d\n", restart);
  auto t0 = std::chrono::steady_clock::now();
  int timestep = restart >= 0 ? restart : 0;
  for (int i = restart >= 0 ? restart * p.ninterm : 0; i <= p.ntot; i++) {
    if (torques && (rc = fargo_update_log(ctx, timestep)) != FARGO_OK) break;
    if (p.ninterm > 0 && (i / p.ninterm) * p.ninterm == i) {
      timestep = i / p.ninterm;
      std::printf("\n*** OUTPUT %d ***\n", i / p.ninterm);
      if ((rc = fargo_write_outputs(ctx, i / p.ninterm)) != FARGO_OK) break;
    }
    if ((rc = fargo_step_DT(ctx, nullptr)) != FARGO_OK) break;
  }
  auto t1 = std::chrono::steady_clock::now();
  if (rc != FARGO_OK) std::fprintf(stderr, "stopped: %s\n", fargo_last_error(ctx));
  std::printf("%g\n", std::chrono::duration<double>(t1 - t0).count());
  fargo_ctx_destroy(ctx);
  return rc == FARGO_OK ? 0 : 1;
}
