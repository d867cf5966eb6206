/* Host stand-in for the CUDA runtime header (see cuda.h beside it): the
 * allocation, copy and synchronisation calls of the reference GPU drivers'
 * main(), declared so the drivers compile; none of them is called. */
#pragma once
#include <stddef.h>
typedef int cudaError_t;
enum cudaMemcpyKind { cudaMemcpyHostToDevice = 1, cudaMemcpyDeviceToHost = 2 };
#ifdef __cplusplus
extern "C" {
#endif
cudaError_t cudaMalloc(void **p, size_t n);
cudaError_t cudaMemcpy(void *dst, const void *src, size_t n, enum cudaMemcpyKind k);
cudaError_t cudaDeviceSynchronize(void);
#ifdef __cplusplus
}
template <class T> static inline cudaError_t cudaMalloc(T **p, size_t n) { return cudaMalloc((void **)p, n); }
#endif
