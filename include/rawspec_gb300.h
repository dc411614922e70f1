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
  RAWSPEC_GB300_K_LARGE_FUSED = 8, /* persistent fused four-step kernel       */
  RAWSPEC_GB300_K_TC = 9,       /* tensor-core DFT product kernel             */
  RAWSPEC_GB300_K_MERGE = 10,   /* compensated integration across buffers     */
  RAWSPEC_GB300_K_COUNT = 11
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

/* The context's CUDA stream (cudaStream_t).  Every call's work is ordered on
 * it: the products' kernels run on per-product streams that fork from it and
 * join back into it, so an event recorded on it brackets a whole buffer. */
void *rawspec_gb300_stream(rawspec_context *ctx);

/* Device pointer and size of the device input buffer
 * ([channel][Nb*Ntpb][pol][re,im] bytes). */
void *rawspec_gb300_device_input(rawspec_context *ctx, size_t *bytes);

/* Enables (1) or disables (0) per-kernel CUDA-event timing.  While enabled,
 * the products run one after another on the context stream, so that each
 * kernel's events time it alone on the GPU. */
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

/* Kernel class that computes product `product` of an initialised context:
 * RAWSPEC_GB300_K_SMALL, RAWSPEC_GB300_K_TC, RAWSPEC_GB300_K_LARGE_FUSED or
 * RAWSPEC_GB300_K_LARGE_A (the two-kernel four-step path); -1 if the
 * context is not initialised or has no such product. */
int rawspec_gb300_product_kernel(rawspec_context *ctx, int product);

/* Kernel choices of one entry of the tuning table (RAWSPEC_GB300_TUNE_FILE,
 * format in rawspec_gb300/csrc/tune.c); -1 (dft) or 0 (the others) leaves
 * the library's own choice. */
typedef struct {
  int dft;   /* N <= 4096: 1 tensor-core DFT (k_tc, where supported), 0 CUDA cores (k_small) */
  int ctas;  /* CTAs per SM that the chunking of k_small / k_large_a/b aims for (default 4) */
  int lag;   /* k_large_fused: the row tiles of slab s follow the column tiles of slab s + lag */
  int ring;  /* k_large_fused: intermediate slabs (> lag) */
} rawspec_gb300_tune;

/* Looks (nfft, nbits, npolout) up in the tuning table named by
 * RAWSPEC_GB300_TUNE_FILE, read at each call; nbits is the width of the
 * samples the kernels read (4-bit input is expanded to 8).  Returns 1 and
 * fills *t if the table has the entry, 0 if it has not or no table is named
 * (*t then holds the unset values), -1 if the file cannot be read.  Used
 * by rawspec_initialize and the device-memory estimate; no CUDA calls. */
int rawspec_gb300_tune_lookup(unsigned nfft, int nbits, int npolout, rawspec_gb300_tune *t);

/* One input buffer of each of n initialised contexts on one device, already
 * copied to the device (rawspec_copy_blocks_to_gpu): the work that
 * rawspec_start_processing(ctxs[k], fft_dirs[k]) queues for each, except that
 * the fused small-FFT kernel launches (FFT lengths up to 4096 on the CUDA
 * cores) of the contexts that share a kernel configuration (FFT length,
 * sample format, polarisations, output mode) run as one grid of up to 8
 * launches.  Each context's dumps, callbacks and integration state are its
 * own, as with separate calls; a context appears at most once.  Contexts on
 * different devices or with profiling on are processed one after another.
 * 0 on success, 1 on error. */
int rawspec_gb300_start_processing_group(rawspec_context *const *ctxs, const int *fft_dirs, int n);

/* Kernel launches of this context that also carried other contexts'
 * buffers (rawspec_gb300_start_processing_group). */
unsigned long long rawspec_gb300_shared_launches(rawspec_context *ctx);

/* ---- channel shards: one observation over several GPUs -------------------
 * A shard is the range [k0, k0 + nk) of channels-within-antenna of every
 * antenna (channel c of antenna a is a * Nc/Nant + c in the GUPPI block), so
 * that all antennas of a channel, which the incoherent sum combines, stay on
 * one GPU; shards exchange nothing.  One process per GPU runs a context of
 * Nant * nk channels for its shard.  Host code only (no CUDA calls). */

/* Shard `rank` of `world` of Nc channels in Nant antennas: nearly equal
 * contiguous ranges of the Nc/Nant channels-within-antenna.  0 on success,
 * 1 on invalid arguments or an empty shard (world > Nc/Nant). */
int rawspec_gb300_shard_range(unsigned int Nc, unsigned int Nant, int rank, int world,
                              unsigned int *k0, unsigned int *nk);

/* Fills *shard with the client fields of *full for shard `rank` of `world`
 * (Nc = Nant * nk, channel batching off, library-allocated host blocks; the
 * weights pointer and the dump callback are shared).  The caller then calls
 * rawspec_initialize(shard).  0 on success, 1 on invalid arguments. */
int rawspec_gb300_shard_context(const rawspec_context *full, int rank, int world,
                                rawspec_context *shard);

/* Copies the shard's channels of one host block of the full observation
 * (Nc channels of channel_bytes each) into a host block of the shard
 * context.  0 on success, 1 on invalid arguments. */
int rawspec_gb300_shard_fill_block(const void *full_block, unsigned int Nc, unsigned int Nant,
                                   unsigned int k0, unsigned int nk, size_t channel_bytes,
                                   void *shard_block);

/* Puts one dump of a shard into the dump buffer of the full observation:
 * rows = Nd * |Npolout| rows of channels, Nt floats per channel; ics = 0 for
 * h_pwrbuf ([rows][Nc][Nt] in the full buffer), 1 for h_icsbuf
 * ([rows][Nc/Nant][Nt]).  0 on success, 1 on invalid arguments. */
int rawspec_gb300_shard_place_dump(const float *shard_dump, unsigned int Nc, unsigned int Nant,
                                   unsigned int k0, unsigned int nk, unsigned int rows,
                                   unsigned int Nt, int ics, float *full_dump);

/* Device memory rawspec_initialize() would allocate for this context (the
 * same validation and kernel configuration, nothing allocated; the context
 * itself is not modified).  Needs the CUDA device gpu_index.  0 on success,
 * 1 if the context is invalid. */
int rawspec_gb300_device_bytes_estimate(const rawspec_context *ctx, size_t *bytes);

/* Allocation-free computation of one output product for one device-resident
 * input buffer.  No counterpart in the reference library.
 *
 * For callers that cannot allocate device memory: a streaming pipeline thread
 * that must never stall (cudaMalloc and cudaFree synchronise the whole device,
 * blocking every other stream), or a host framework that hands out all device
 * memory from its own pool and budget.  The caller passes the input and the
 * output; the function calls no cudaMalloc, cudaFree or other allocating
 * routine and needs no rawspec_initialize().
 *
 *   d_in     device input, [Nc][samples_per_channel][Np][re,im], Nbps = 8 or
 *            16 bits per component (the layout rawspec_copy_blocks_to_gpu
 *            produces; 4-bit input must be expanded first), aligned to one
 *            time sample (Np * 2 * Nbps / 8 bytes)
 *   Nt, Na   FFT length (power of two, at most 4096) and spectra per
 *            integration; Nt*Na must divide samples_per_channel
 *   Npolout  1, +4 (full pol) or -4 (Stokes; +4 and -4 need Np == 2)
 *   d_out    device output, [Nd][|Npolout|][Nc][Nt] float, FFT-shifted, with
 *            Nd = samples_per_channel / (Nt*Na): the same values
 *            rawspec_start_processing() dumps for such a product
 *   stream   cudaStream_t to queue the work on (0 = legacy default stream)
 *
 * Scratch: a file-scope device array of 4 MiB of partial sums plus a 4096-entry
 * twiddle table (4.03 MiB), held by every GPU that loads the library until the
 * process exits.  The partial-sum split is limited to what fits; FFT lengths
 * above 4096 are rejected with an error.  The first call on a device looks up
 * the array's device address (make that first call before any stream capture
 * on that device).  Every call shares the array and it keeps the last call's
 * contents; everything a call reads from it is written by the same call first.
 * The looked-up address belongs to the device's primary context (the CUDA
 * runtime's); after cudaDeviceReset the library must be reloaded before this
 * entry point is used again.
 * Calls that overlap on the GPU (different streams, or another host thread)
 * race on the array and must be serialised by the caller.
 * Returns 0 when the work is queued, 1 on invalid arguments or a CUDA error
 * (message on stderr). */
int rawspec_gb300_product_noalloc(const void *d_in, unsigned int Nc, unsigned int Np,
                                  unsigned int Nbps,
                                  unsigned long long samples_per_channel,
                                  unsigned int Nt, unsigned int Na, int Npolout,
                                  int fft_dir, int input_conjugated,
                                  float *d_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* RAWSPEC_GB300_EXT_H */
