/* A driver shaped like the reference's UH-GPU/<case>/<n>pt_main.cpp: it
 * cudaMallocs two padded grids, fills every cell with rand() % 50, builds the
 * two MLIR memref descriptors, calls the program's generated C-interface entry
 * and copies the result back.  Here the entry is the backend's wrapper
 * (uxxxxxxxxh_gb300.ciface); the result grid is written to argv[2] for the
 * test to compare with the oracle.  Usage: mlir_driver Z Y X out.bin
 * (Z = 1 for a rank-2 program). */
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <cuda_runtime.h>

typedef struct {
    double *allocated, *aligned;
    int64_t offset, sizes[3], strides[3];
} memref3;
typedef struct {
    double *allocated, *aligned;
    int64_t offset, sizes[2], strides[2];
} memref2;

extern void UHS_ENTRY(void *a, void *b);

int main(int argc, char **argv) {
    if (argc != 5) return 2;
    const int64_t M = atoll(argv[1]), N = atoll(argv[2]), Q = atoll(argv[3]);
    const size_t n = (size_t)(M * N * Q);
    double *h = (double *)malloc(n * sizeof(double));
    for (size_t i = 0; i < n; ++i) h[i] = rand() % 50;
    double *a, *b;
    if (cudaMalloc((void **)&a, n * sizeof(double)) || cudaMalloc((void **)&b, n * sizeof(double))) return 3;
    cudaMemcpy(a, h, n * sizeof(double), cudaMemcpyHostToDevice);
    cudaMemcpy(b, h, n * sizeof(double), cudaMemcpyHostToDevice); /* both halos set */
    if (M == 1) {
        memref2 A = {a, a, 0, {N, Q}, {Q, 1}}, B = {b, b, 0, {N, Q}, {Q, 1}};
        UHS_ENTRY(&A, &B);
    } else {
        memref3 A = {a, a, 0, {M, N, Q}, {N * Q, Q, 1}}, B = {b, b, 0, {M, N, Q}, {N * Q, Q, 1}};
        UHS_ENTRY(&A, &B);
    }
    cudaDeviceSynchronize();
    cudaMemcpy(h, a, n * sizeof(double), cudaMemcpyDeviceToHost);
    FILE *f = fopen(argv[4], "wb");
    fwrite(h, sizeof(double), n, f);
    fclose(f);
    return 0;
}
