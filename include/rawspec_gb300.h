/*
 * rawspec_gb300.h -- extensions of the GB300-native librawspec beyond the
 * reference C interface (rawspec.h).  None of these is needed by a client of
 * the reference API; they serve instrumentation, host-only validation and
 * tests.  No entry point here has a counterpart in the reference library.
 */
#ifndef RAWSPEC_GB300_EXT_H
#define RAWSPEC_GB300_EXT_H

#include "rawspec.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Kernel classes for the profiling counters. */
enum rawspec_gb300_kernel_class {
  RAWSPEC_GB300_K_SMALL = 0,    /* fused unpack/FFT/detect/integrate, N <= 4096 */
  RAWSPEC_GB300_K_FINALIZE = 1, /* fixed-order sum of per-chunk partials      */
  RAWSPEC_GB300_K_LARGE_A = 2,  /* four-step pass A (column FFTs)             */
  RAWSPEC_GB300_K_LARGE_B = 3,  /* four-step pass B (row FFTs + detection)    */
  RAWSPEC_GB300_K_ICS = 4,      /* weighted incoherent sum                    */
  RAWSPEC_GB300_K_EXPAND4 = 5,  /* 4-bit expansion                            */
  RAWSPEC_GB300_K_D2H = 6,      /* dump copies device -> host                 */
  RAWSPEC_GB300_K_H2D = 7,      /* block copies host -> device                */
  RAWSPEC_GB300_K_COUNT = 8
};

/* Validates and normalises a context exactly as rawspec_initialize() does
 * (Npolout, Nbps, Ntmax, Nb, Nb_host, Nant, Nbc, Nds, h_pwrbuf_size) without
 * touching CUDA or allocating anything.  0 on success, 1 on error. */
int rawspec_gb300_validate(rawspec_context *ctx);

/* Derived per-product quantities of a validated context: spectra per buffer
 * (Nss), buffers per dump (Nis), spectra per dump (Nd).  0 on success. */
int rawspec_gb300_product_info(const rawspec_context *ctx, int product,
                               unsigned int *Nss, unsigned int *Nis,
                               unsigned int *Nd);

/* The CUDA stream (cudaStream_t) all work of the context is queued on. */
void *rawspec_gb300_stream(rawspec_context *ctx);

/* Device pointer and size of the device input buffer
 * ([channel][Nb*Ntpb][pol][re,im] bytes). */
void *rawspec_gb300_device_input(rawspec_context *ctx, size_t *bytes);

/* Enables (1) or disables (0) per-kernel CUDA-event timing. */
int rawspec_gb300_set_profiling(rawspec_context *ctx, int enable);

/* Waits for the stream, then returns the accumulated device time (ms) and
 * the number of launches of a kernel class since the last reset. */
int rawspec_gb300_profile(rawspec_context *ctx, int kernel_class,
                          double *total_ms, unsigned long long *launches);

/* Clears the profiling counters. */
int rawspec_gb300_reset_profile(rawspec_context *ctx);

/* Number of this library's kernels launched on the context so far. */
unsigned long long rawspec_gb300_kernel_launches(rawspec_context *ctx);

/* Bytes of device memory held by the context. */
size_t rawspec_gb300_device_bytes(rawspec_context *ctx);

#ifdef __cplusplus
}
#endif

#endif /* RAWSPEC_GB300_EXT_H */
