// stand-in for cufft.h in the CPU build of the reference: the Z2Z calls it makes
// (src/Main.cu:191-199, src/SgMain.cu:117-161) run on the oracle's FFT
#pragma once
typedef struct {
  double x, y;
} cufftDoubleComplex;
typedef int cufftHandle;
typedef int cufftResult;
enum { CUFFT_SUCCESS = 0, CUFFT_INVALID_PLAN = 1 };
#define CUFFT_Z2Z 0x69
#define CUFFT_FORWARD (-1)
#define CUFFT_INVERSE 1
cufftResult cufftPlan2d(cufftHandle *plan, int nx, int ny, int type);
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex *in, cufftDoubleComplex *out, int direction);
cufftResult cufftDestroy(cufftHandle plan);
