/* Host stand-in for the CUDA driver header, used only to compile the
 * reference's GPU drivers for their CPU loop (cpu_verify).  It declares the
 * handful of driver calls the drivers' main() makes, with the three-argument
 * context call those drivers were written against; none of them is called. */
#pragma once
typedef struct uhs_shim_ctx *CUcontext;
typedef struct uhs_shim_mod *CUmodule;
typedef int CUdevice;
typedef int CUresult;
#ifdef __cplusplus
extern "C" {
#endif
CUresult cuInit(unsigned int flags);
CUresult cuDeviceGet(CUdevice *dev, int ordinal);
CUresult cuCtxCreate(CUcontext *ctx, unsigned int flags, CUdevice dev);
#ifdef __cplusplus
}
#endif
