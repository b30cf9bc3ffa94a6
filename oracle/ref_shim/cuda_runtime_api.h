/*
 * cuda_runtime_api.h -- CPU stand-in for the three CUDA runtime calls the
 * reference's AProductCore.cpp makes (cudaMalloc, cudaMemcpy, cudaFree).
 * "Device" memory is host memory; cudaFree releases a pointer once, so the
 * reference's second cudaFree(ADev) (AProductCore.cpp:540-541) is harmless.
 * Used only to build the reference's sources into the checker binary.
 */
#ifndef ORACLE_REF_SHIM_CUDA_RUNTIME_API_H_
#define ORACLE_REF_SHIM_CUDA_RUNTIME_API_H_

#include <stddef.h>

typedef int cudaError_t;
enum cudaMemcpyKind { cudaMemcpyHostToHost = 0, cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2, cudaMemcpyDeviceToDevice = 3 };

cudaError_t cudaMalloc(void** ptr, size_t size);
cudaError_t cudaMemcpy(void* dst, const void* src, size_t count, enum cudaMemcpyKind kind);
cudaError_t cudaFree(void* ptr);

#endif
