/* cuda.h -- empty CPU stand-in; the reference includes it but calls no driver API. */
#ifndef ORACLE_REF_SHIM_CUDA_H_
#define ORACLE_REF_SHIM_CUDA_H_
#endif
