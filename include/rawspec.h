/*
 * rawspec.h -- drop-in C interface of the GB300-native librawspec.
 *
 * This header declares the same context structure (same members, same order,
 * same types, hence the same ABI) and the same twelve entry points as the
 * reference library's public header (rawspec.h:32-148 for the structure,
 * rawspec.h:161-234 for the prototypes), so that the reference CLI
 * (rawspec.c) and its SIGPROC/FBH5/UDP writers compile and link against this
 * library unchanged.  The text below is this project's own; only the names,
 * the member layout, the constants and the signatures are kept identical,
 * because a client compiled against either header must see the same ABI.
 *
 * Semantics that differ from the reference are listed in the comments of the
 * affected members and functions (each difference keeps the reference's
 * results and only removes a hazard of the reference implementation).
 */
#ifndef RAWSPEC_GB300_RAWSPEC_H
#define RAWSPEC_GB300_RAWSPEC_H

#include <stddef.h>
#include <unistd.h>   /* off_t */

/* fft_dir argument of rawspec_start_processing(): > 0 forward
 * (exp(-2 pi i k n / N)), <= 0 inverse (exp(+2 pi i k n / N)).  Neither
 * direction is normalised. */
#define RAWSPEC_FORWARD_FFT (+1)
#define RAWSPEC_INVERSE_FFT (-1)

/* Maximum number of simultaneous output products per context. */
#define MAX_OUTPUTS (4)

/* Size in bytes of one GUPPI RAW block as seen by the context: channels x
 * time samples x polarisations x 2 components x bits per component / 8. */
#define RAWSPEC_BLOCSIZE(pctx) \
  (((pctx)->Nc * (pctx)->Ntpb * (pctx)->Np * 2 * (pctx)->Nbps) / 8)

/* callback_type values passed to the dump callback. */
#define RAWSPEC_CALLBACK_PRE_DUMP  (0)
#define RAWSPEC_CALLBACK_POST_DUMP (1)

typedef struct rawspec_context_s rawspec_context;

/* Dump callback.  Called on a CUDA host-function thread, in stream order:
 * PRE_DUMP before the library writes h_pwrbuf[output_product] (and
 * h_icsbuf[output_product]) for a dump, POST_DUMP once both are complete.
 * The callback must not call CUDA. */
typedef void (*rawspec_dump_callback_t)(rawspec_context *ctx,
                                        int output_product,
                                        int callback_type);

struct rawspec_context_s {
  /* ---- set by the client ---------------------------------------------- */
  unsigned int No;        /* output products, 1..MAX_OUTPUTS                */
  unsigned int Np;        /* input polarisations, 1 or 2                    */
  unsigned int Nant;      /* antennas; Nc is a multiple of Nant (0 -> 1)    */
  unsigned int Nc;        /* coarse channels per block                      */
  unsigned int Ntpb;      /* time samples per block                         */
  unsigned int exit_soon; /* set by clients' writers; returned by wait      */

  /* Coarse channels per batch.  Accepted for compatibility (0, 1 = auto,
   * or a divisor of Nc) and normalised exactly as the reference does, but
   * this library keeps full-Nc state on the device and does not need to
   * batch; the value only affects what is printed and stored back. */
  unsigned int Nbc;

  /* Bits per component: 4, 8 or 16 (0 means 8).  4-bit input (high nibble
   * real, low nibble imaginary) is stored back as 8 by rawspec_initialize(),
   * as clients expect; the host blocks are then sized for 8 bits. */
  unsigned int Nbps;

  /* Per product output polarisation mode: 1 total power; +4 full pol
   * (XX, YY, Re XY*, Im XY*); -4 full Stokes (I, Q, U, V).  Anything else,
   * or Np != 2, is coerced to 1 by rawspec_initialize(). */
  int Npolout[MAX_OUTPUTS];

  /* Per product FFT length (fine channels per coarse channel).  Every Nts
   * value must divide the largest one (Ntmax). */
  unsigned int Nts[MAX_OUTPUTS];

  /* Per product integration length in spectra.  Nts[i]*Nas[i] must either
   * divide Nb*Ntpb or be a multiple of it. */
  unsigned int Nas[MAX_OUTPUTS];

  rawspec_dump_callback_t dump_callback;
  void *user_data;        /* untouched by the library                       */

  unsigned int Nb;        /* blocks per GPU input buffer (0 = Ntmax/Ntpb)    */
  unsigned int Nb_host;   /* host block buffers (0 = Nb)                     */

  /* Host block buffers.  NULL: allocated (pinned) by the library.  Otherwise
   * an array of Nb_host caller-owned blocks that the library page-locks
   * while the context lives. */
  char **h_blkbufs;

  int gpu_index;          /* CUDA device ordinal                             */
  int input_conjugated;   /* 1: negate Im XY* / Stokes V (flipped band)      */
  int incoherently_sum;   /* 1: also produce the weighted antenna sum        */
  int Naws;               /* number of weights in Aws: 1 or Nant             */
  float *Aws;             /* antenna weights (caller-owned; never freed)     */

  /* ---- set by the library --------------------------------------------- */
  /* Integrated, FFT-shifted spectra of the latest dump of each product,
   * laid out [Nds][|Npolout|][Nc][Nts] as float (pinned host memory). */
  float *h_pwrbuf[MAX_OUTPUTS];
  size_t h_pwrbuf_size[MAX_OUTPUTS];

  /* Weighted incoherent sums, [Nds][|Npolout|][Nc/Nant][Nts] float, when
   * incoherently_sum is 1 (size h_pwrbuf_size[i] / Nant). */
  float *h_icsbuf[MAX_OUTPUTS];

  unsigned int Nds[MAX_OUTPUTS]; /* spectra per dump                        */

  unsigned int Ntmax;     /* largest Nts value                               */
  void *gpu_ctx;          /* library-private state                           */
};

/* Output modes used by the reference CLI's writers. */
typedef enum {
  RAWSPEC_FILE,
  RAWSPEC_NET
} rawspec_output_mode_t;

#ifdef __cplusplus
extern "C" {
#endif

/* Library version string. */
const char *get_librawspec_version();

/* FFT implementation string.  This library has no cuFFT dependency; the
 * string names the native FFT instead. */
const char *get_cufft_version();

/* Validates and normalises the context, derives Ntmax/Nb/Nb_host/Nds,
 * allocates host and device buffers and creates the processing stream.
 * Returns 0 on success, non-zero on error (a message goes to stderr). */
int rawspec_initialize(rawspec_context *ctx);

/* Releases everything rawspec_initialize() acquired.  Caller-owned memory
 * (caller h_blkbufs, Aws) is not freed. */
void rawspec_cleanup(rawspec_context *ctx);

/* Copies num_blocks host blocks, starting at h_blkbufs[src_idx % Nb_host],
 * into the device input buffer starting at block dst_idx % Nb.  Returns
 * once the host blocks may be reused.  0 on success. */
int rawspec_copy_blocks_to_gpu(rawspec_context *ctx,
                               off_t src_idx, off_t dst_idx, size_t num_blocks);

/* Same, for packed 4-bit complex host blocks (one byte per complex sample:
 * high nibble real, low nibble imaginary, both two's complement). */
int rawspec_copy_blocks_to_gpu_expanding_complex4(rawspec_context *ctx,
                                                  off_t src_idx, off_t dst_idx,
                                                  size_t num_blocks);

/* Zeroes num_blocks device blocks starting at dst_idx % Nb (wrapping). */
int rawspec_zero_blocks_to_gpu(rawspec_context *ctx,
                               off_t dst_idx, size_t num_blocks);

/* Queues the processing of the device input buffer: FFT, detection,
 * integration and, where an integration completes, the dump to h_pwrbuf
 * with PRE/POST callbacks.  Asynchronous; 0 on success. */
int rawspec_start_processing(rawspec_context *ctx, int fft_dir);

/* rawspec_copy_blocks_to_gpu(ctx, 0, 0, num_blocks) (or the 4-bit variant)
 * followed by rawspec_start_processing(ctx, fft_dir). */
int rawspec_copy_blocks_to_gpu_and_start_processing(rawspec_context *ctx,
                                                    size_t num_blocks,
                                                    char expand4bps_to8bps,
                                                    int fft_dir);

/* Waits for pending work, clears every integration and resets the buffer
 * counter.  0 on success. */
int rawspec_reset_integration(rawspec_context *ctx);

/* 1 when the processing stream is idle, else 0 (the reference returns the
 * same 0/1 values). */
unsigned int rawspec_check_for_completion(rawspec_context *ctx);

/* Queues one PRE_DUMP callback per product, waits for the stream, and
 * returns ctx->exit_soon (non-zero also on a CUDA error). */
int rawspec_wait_for_completion(rawspec_context *ctx);

#ifdef __cplusplus
}
#endif

#endif /* RAWSPEC_GB300_RAWSPEC_H */
