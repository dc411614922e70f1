/* rawspec_gb300_io.h -- the callers either side of the spectrometer path:
 * GUPPI RAW ingest (headers, packet-index gaps, block streaming into a
 * rawspec context) and SIGPROC filterbank output of the dumps.
 *
 * Host-side C, exported from librawspec.so beside the rawspec.h interface.
 * Each declaration names the reference code whose behaviour it restates. */
#ifndef RAWSPEC_GB300_IO_H
#define RAWSPEC_GB300_IO_H

#include <stddef.h>
#include <stdint.h>
#include <sys/types.h>

#include "rawspec.h"

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------------------
 * GUPPI RAW headers
 * ------------------------------------------------------------------------- */

/* Largest header read (a multiple of 80 and 512 bytes). */
#define RAWSPEC_GB300_RAW_MAX_HDR 25600

/* The observation parameters of one RAW block header (the fields of the
 * reference's rawspec_raw_hdr_t, rawspec_rawutils.h:7-28). */
typedef struct {
  int directio;
  size_t blocsize;
  unsigned int npol;      /* NPOL 4 (cross products) is reported as 2 */
  unsigned int obsnchan;
  unsigned int nbits;
  int64_t pktidx;         /* -1 if absent */
  double obsfreq, obsbw, tbin;
  double ra;              /* hours */
  double dec;             /* degrees */
  double mjd;
  int beam_id, nbeam, refbeam;
  unsigned int nants;
  char src_name[81];
  char telescop[81];
  off_t hdr_pos;          /* file offset of the header */
  size_t hdr_size;        /* header bytes up to END, without DIRECTIO padding */
} rawspec_gb300_raw_hdr;

/* Parses the header cards in buf[0..len) (80-byte "KEYWORD = value" cards up
 * to END) into hdr, with the reference's defaults for absent keywords
 * (rawspec_rawutils.c:175-216).  Returns 0. */
int rawspec_gb300_raw_parse_header(const char *buf, size_t len, rawspec_gb300_raw_hdr *hdr);

/* Bytes from the start of the header to just after its END card, plus the
 * DIRECTIO padding to a 512-byte boundary when directio is set; 0 if no END
 * card is found (rawspec_rawutils.c:154-172). */
size_t rawspec_gb300_raw_header_size(const char *buf, size_t len, int directio);

/* Reads and parses the header at the current offset of fd and leaves fd at
 * the start of the block's data.  Returns that offset, 0 at end of file, or
 * -1 on an error or a missing required keyword (rawspec_rawutils.c:222-261). */
off_t rawspec_gb300_raw_read_header(int fd, rawspec_gb300_raw_hdr *hdr);

/* Sexagesimal "[+-]dd:mm:ss.s" (or a plain number) to decimal
 * (rawspec_rawutils.c:112-152). */
double rawspec_gb300_raw_dms_to_decimal(const char *dms);

/* ---------------------------------------------------------------------------
 * Packet-index sequencing (rawspec.c:600-605, 913-971)
 * ------------------------------------------------------------------------- */

typedef struct {
  int started;
  int64_t prev;   /* packet index of the previous block (or missing block) */
  int64_t step;   /* expected increment, learnt from the first increase */
} rawspec_gb300_pktidx_state;

enum {
  RAWSPEC_GB300_PKT_TAKE = 0,       /* take the block, after *nfill zero blocks */
  RAWSPEC_GB300_PKT_END_FILE = 1,   /* repeated index: the rest of this file is skipped */
  RAWSPEC_GB300_PKT_BACKWARD = 2,   /* index went backwards: the stem ends */
  RAWSPEC_GB300_PKT_MISALIGNED = 3  /* jump not a multiple of the step: the stem ends */
};

/* Classifies the next block's packet index; on TAKE, *nfill is the number of
 * missing blocks to fill with zeros before it and the state advances. */
int rawspec_gb300_pktidx_step(rawspec_gb300_pktidx_state *st, int64_t pktidx, int64_t *nfill);

/* ---------------------------------------------------------------------------
 * Streaming ingest
 * ------------------------------------------------------------------------- */

/* Sets ctx->Nc, Np, Nbps, Ntpb, Nant and input_conjugated from a block header
 * for the channels [schan, schan + nchan) (nchan 0: all channels), as the
 * reference CLI derives them (rawspec.c:613-745 without antenna selection);
 * *expand4 is set for 4-bit input.  Returns 0, or 1 for an invalid channel
 * range or block geometry. */
int rawspec_gb300_ingest_geometry(const rawspec_gb300_raw_hdr *hdr, unsigned int schan, unsigned int nchan,
                                  rawspec_context *ctx, int *expand4);

typedef struct {
  long long blocks_read;   /* data blocks read from the files */
  long long blocks_zero;   /* zero blocks put in for missing packet indices */
  long long buffers;       /* buffers handed to the GPU */
  int stop;                /* 0, or the RAWSPEC_GB300_PKT_* reason that ended the stem, or -1: read error */
} rawspec_gb300_ingest_stats;

/* Streams the files of one stem, in order, through an initialised context
 * whose geometry matches them (rawspec_gb300_ingest_geometry): reads each
 * block's channels [schan, schan + ctx->Nc) into the host blocks, puts in
 * zero blocks for missing packet indices, and hands every complete buffer to
 * the GPU with rawspec_wait_for_completion +
 * rawspec_copy_blocks_to_gpu_and_start_processing (rawspec.c:906-1032);
 * waits for completion at the end.  An incomplete last buffer is not
 * processed.  Returns 0, or 1 on an error of the library. */
int rawspec_gb300_ingest_files(rawspec_context *ctx, const char *const *paths, int npaths, unsigned int schan,
                               int expand4, rawspec_gb300_ingest_stats *stats);

/* The same as a reusable handle, for a context that streams several stems:
 * open allocates a second set of pinned host blocks (the file reads of one
 * buffer overlap the host-to-device copy of the previous one, the context's
 * block pointers being switched per buffer and restored at the end of each
 * stem) and the reader threads; NULL on failure.  rawspec_gb300_ingest_files
 * is open + stem + close. */
typedef struct rawspec_gb300_ingest rawspec_gb300_ingest;
rawspec_gb300_ingest *rawspec_gb300_ingest_open(rawspec_context *ctx, int expand4);
int rawspec_gb300_ingest_stem(rawspec_gb300_ingest *ingest, const char *const *paths, int npaths, unsigned int schan,
                              rawspec_gb300_ingest_stats *stats);
void rawspec_gb300_ingest_close(rawspec_gb300_ingest *ingest);

/* ---------------------------------------------------------------------------
 * SIGPROC filterbank output
 * ------------------------------------------------------------------------- */

/* Filterbank header fields (the reference's fb_hdr_t, rawspec_fbutils.h:68-117). */
typedef struct {
  int machine_id, telescope_id, data_type, barycentric, pulsarcentric;
  double src_raj;   /* hours */
  double src_dej;   /* degrees */
  double az_start, za_start, fch1, foff;
  int nchans, nbeams, ibeam, nbits;
  double tstart, tsamp;
  int nifs;
  char source_name[81];
  char rawdatafile[81];
  int nfpc, refbeam;
} rawspec_gb300_fil_hdr;

/* Serialises a SIGPROC header (HEADER_START ... HEADER_END, little-endian,
 * the reference's keyword order, rawspec_fbutils.c:246-322) into buf.
 * Returns the number of bytes, or -1 if cap is too small. */
long rawspec_gb300_fil_header(const rawspec_gb300_fil_hdr *hdr, void *buf, size_t cap);

/* The same header padded to at least minlen bytes with blank "rawdatafile"
 * entries ahead of the real one (rawspec_fbutils.c:330-404); minlen 0: no
 * padding. */
long rawspec_gb300_fil_header_padded(const rawspec_gb300_fil_hdr *hdr, void *buf, size_t cap, int minlen);

/* SIGPROC telescope_id of a telescope name, -1 if unknown
 * (rawspec_fbutils.c:533-576). */
int rawspec_gb300_telescope_id(const char *name);

/* The header of output product `product` for a stem whose first block header
 * is raw, processing channels from schan (rawspec.c:484-492, 800-826). */
int rawspec_gb300_fil_header_for_product(const rawspec_gb300_raw_hdr *raw, const rawspec_context *ctx, int product,
                                         unsigned int schan, const char *rawdatafile, rawspec_gb300_fil_hdr *out);

/* Most antennas a writer splits one product into. */
#define RAWSPEC_GB300_MAX_FIL_FILES 64

/* One output product's filterbank files: <dest>/<basename(stem)>.rawspec.NNNN.fil
 * (or one file per antenna, "<stem>-antAAA", when the context has several
 * antennas and per_antenna is set or the antennas are not summed), plus the
 * incoherent sum's file under ics_stem when the context sums antennas
 * (rawspec_file.c:15-100, rawspec.c:624-627). */
typedef struct rawspec_gb300_fil_writer rawspec_gb300_fil_writer;

/* Opens the product's files and writes their headers; NULL on failure. */
rawspec_gb300_fil_writer *rawspec_gb300_fil_writer_open(const rawspec_context *ctx, int product,
                                                        const rawspec_gb300_fil_hdr *hdr, const char *dest,
                                                        const char *stem, int output_idx, int per_antenna,
                                                        const char *ics_stem);

/* Waits for a pending write, closes the files and frees the writer; returns
 * 0, or 1 if a write or a close failed. */
int rawspec_gb300_fil_writer_close(rawspec_gb300_fil_writer *w);

/* A dump callback for rawspec_context.dump_callback.  ctx->user_data points to
 * an array of writer pointers indexed by output product.  PRE_DUMP waits for
 * the product's previous write; POST_DUMP starts a writer thread that writes
 * the dump (the whole buffer for one antenna; per spectrum, polarisation and
 * antenna slices for split files; the incoherent sum to its file), so that
 * file I/O overlaps the next buffer's processing (rawspec_file.c:102-243).
 * A failed write sets ctx->exit_soon. */
void rawspec_gb300_fil_dump_callback(rawspec_context *ctx, int output_product, int callback_type);

/* ---------------------------------------------------------------------------
 * UDP output of the dumps (rawspec_socket.c:21-354)
 * ------------------------------------------------------------------------- */

/* A UDP socket connected to host:port (IPv4), with the don't-fragment probe
 * option; -1 if the address cannot be resolved or connected, or if the path's
 * MTU is below 8600 bytes (the packets carry up to 8 KiB of data). */
int rawspec_gb300_net_open(const char *host, const char *port);

/* Output rates of the products, total_gbps shared in proportion to their data
 * volume, i.e. to 1/Nas[i] (rawspec.c:884-901). */
void rawspec_gb300_net_rates(const rawspec_context *ctx, double total_gbps, double *rates_gbps);

/* One output product's UDP sender: each dump is cut into packets of at most
 * 2048 floats (whole spectra when a spectrum has fewer channels), each
 * behind a SIGPROC header of its own channel count, first channel frequency
 * and start time, padded so that the data start on a 512-byte boundary of a
 * packet-socket frame (whose UDP payload begins 0x6c bytes in); packets are
 * paced to rate_gbps.  The dump is sent from the start of h_pwrbuf as Nds
 * spectra of hdr->nchans floats, as the reference does. */
typedef struct rawspec_gb300_net_writer rawspec_gb300_net_writer;
rawspec_gb300_net_writer *rawspec_gb300_net_writer_open(const rawspec_context *ctx, int product,
                                                        const rawspec_gb300_fil_hdr *hdr, int fd,
                                                        double rate_gbps);

typedef struct {
  long long dumps, spectra, packets, bytes, error_packets;
  double seconds;  /* time spent sending, pacing included */
} rawspec_gb300_net_stats;

int rawspec_gb300_net_writer_stats(rawspec_gb300_net_writer *w, rawspec_gb300_net_stats *st);

/* Waits for a dump being sent and frees the writer (the socket stays open);
 * 0, or 1 if packets could not be sent. */
int rawspec_gb300_net_writer_close(rawspec_gb300_net_writer *w);

/* Dump callback (ctx->user_data: array of writer pointers by product):
 * PRE_DUMP waits for the product's previous dump to be sent, POST_DUMP starts
 * a sender thread for this one (rawspec_socket.c:327-354). */
void rawspec_gb300_net_dump_callback(rawspec_context *ctx, int output_product, int callback_type);

#ifdef __cplusplus
}
#endif

#endif /* RAWSPEC_GB300_IO_H */
