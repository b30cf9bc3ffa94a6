/*
 * cufft.h -- CPU stand-in for the slice of the cuFFT API that the
 * reference's AProductCore.cpp calls (cufftPlan3d, cufftExecZ2Z,
 * cufftDestroy; AProductCore.cpp:47, :212-229, :719-739).  Only the public
 * names and signatures match cuFFT; the transform is the oracle's own CPU
 * FFT (oracle/cfft.c).  Used only to build the reference's sources into the
 * checker binary under oracle/_ref.
 */
#ifndef ORACLE_REF_SHIM_CUFFT_H_
#define ORACLE_REF_SHIM_CUFFT_H_

#include "cuda_runtime_api.h"

typedef struct { double x, y; } cufftDoubleComplex;
typedef int cufftHandle;
typedef enum { CUFFT_SUCCESS = 0, CUFFT_INVALID_PLAN = 1, CUFFT_ALLOC_FAILED = 2, CUFFT_INVALID_VALUE = 4 } cufftResult;
typedef enum { CUFFT_Z2Z = 0x69 } cufftType;
#define CUFFT_FORWARD -1
#define CUFFT_INVERSE 1

cufftResult cufftPlan3d(cufftHandle* plan, int nx, int ny, int nz, cufftType type);
cufftResult cufftExecZ2Z(cufftHandle plan, cufftDoubleComplex* idata, cufftDoubleComplex* odata, int direction);
cufftResult cufftDestroy(cufftHandle plan);

#endif
