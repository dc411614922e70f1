/* io_raw.c -- GUPPI RAW ingest: header cards, packet-index sequencing and the
 * streaming of a stem's blocks into a rawspec context.
 *
 * Restates the behaviour of the reference's RAW utilities
 * (rawspec_rawutils.c, whose keyword lookup follows the WCSTools hget
 * conventions) and of the block loop of its CLI (rawspec.c:906-1032), in this
 * project's own code.  Header cards are 80 bytes, "KEYWORD = value", the
 * keyword in the first 8 columns (case-insensitive), the value a quoted
 * string or the text up to a '/' comment; the header ends with an END card,
 * followed (DIRECTIO = 1) by padding to a 512-byte boundary, then the block's
 * data: OBSNCHAN channels of [time][pol][re, im] samples. */
#define _GNU_SOURCE
#include <ctype.h>
#include <errno.h>
#include <fcntl.h>
#include <limits.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include "rawspec_gb300_io.h"

#define RSG_EXPORT __attribute__((visibility("default")))

/* ---------------------------------------------------------------------------
 * Card lookup
 * ------------------------------------------------------------------------- */

/* The value text of the first card whose keyword is `key` (case-insensitive,
 * at most 8 characters, optionally preceded by blanks and followed by '='
 * or a blank), copied into out (up to outlen - 1 characters, surrounding
 * blanks removed, quotes stripped).  Returns 1 if found, 0 if not.  The
 * search stops at the END card. */
static int card_value(const char *buf, size_t len, const char *key, char *out, size_t outlen) {
  const size_t klen = strlen(key);
  for (size_t c = 0; c < len; c += 80) {
    const char *card = buf + c;
    const size_t clen = len - c < 80 ? len - c : 80;
    if (clen >= 4 && strncmp(card, "END ", 4) == 0) return 0;
    /* keyword: leading blanks within the first 8 columns */
    size_t k = 0;
    while (k < 8 && k < clen && card[k] == ' ') ++k;
    if (k >= 8 || k + klen > clen || strncasecmp(card + k, key, klen) != 0) continue;
    const char next = k + klen < clen ? card[k + klen] : ' ';
    if (next != '=' && next > ' ' && next < 127) continue;  /* a longer keyword */
    /* value: quoted string, else the text after '=' up to a '/' comment
     * (column 80 excluded) */
    char line[81];
    memset(line, 0, sizeof(line));
    memcpy(line, card, clen);
    const char *v1, *v2;
    const char *slash = strchr(line, '/');
    const char *q1 = strchr(line, '\'');
    char quote = '\'';
    if (!q1) {
      q1 = strchr(line, '"');
      quote = '"';
    }
    if (q1 && (!slash || q1 < slash)) {
      v1 = q1 + 1;
      const char *q2 = strchr(v1, quote);
      if (!q2) q2 = slash ? slash : line + 79;
      v2 = q2;
    } else {
      const char *eq = strchr(line, '=');
      v1 = eq ? eq + 1 : line + 9;
      v2 = slash ? slash : line + 79;
    }
    while (v1 < v2 && *v1 == ' ') ++v1;
    while (v2 > v1 && (v2[-1] == ' ' || v2[-1] == '\r')) --v2;
    size_t n = (size_t)(v2 - v1);
    if (n >= outlen) n = outlen - 1;
    memcpy(out, v1, n);
    out[n] = '\0';
    if (strcmp(out, "-0") == 0) memmove(out, out + 1, 2);
    return 1;
  }
  return 0;
}

/* Decimal conversion of a numeric value, accepting Fortran 'D' exponents. */
static double value_to_double(const char *v) {
  char tmp[96];
  snprintf(tmp, sizeof(tmp), "%s", v[0] == '#' ? v + 1 : v);
  for (char *p = tmp; *p; ++p)
    if (*p == 'D' || *p == 'd') {
      /* only as an exponent marker: a digit or a sign on each side */
      if (p > tmp && (isdigit((unsigned char)p[-1]) || p[-1] == '.') &&
          (isdigit((unsigned char)p[1]) || p[1] == '+' || p[1] == '-'))
        *p = 'e';
    }
  return strtod(tmp, NULL);
}

/* Signed 32-bit: the value read as a decimal number and truncated towards
 * zero (with a 0.001 guard and saturation), as the reference's lookup does. */
static int32_t get_s32(const char *buf, size_t len, const char *key, int32_t def) {
  char v[96];
  if (!card_value(buf, len, key, v, sizeof(v))) return def;
  const double d = value_to_double(v);
  if (d + 0.001 > (double)INT32_MAX) return INT32_MAX;
  if (d >= 0) return (int32_t)(d + 0.001);
  if (d - 0.001 < (double)INT32_MIN) return INT32_MIN;
  return (int32_t)(d - 0.001);
}

/* Unsigned and 64-bit integers: C integer syntax (decimal, 0x hex, 0
 * octal); a value with trailing non-digits is read as a decimal number. */
static unsigned long long get_ull(const char *buf, size_t len, const char *key, unsigned long long def, int is_signed) {
  char v[96];
  if (!card_value(buf, len, key, v, sizeof(v))) return def;
  const char *s = v[0] == '#' ? v + 1 : v;
  char *end = NULL;
  if (is_signed) {
    const long long x = strtoll(s, &end, 0);
    if (end && *end) return (unsigned long long)(long long)atof(s);
    return (unsigned long long)x;
  }
  const unsigned long long x = strtoull(s, &end, 0);
  if (end && *end) return (unsigned long long)atof(s);
  return x;
}

static double get_dbl(const char *buf, size_t len, const char *key, double def) {
  char v[96];
  if (!card_value(buf, len, key, v, sizeof(v))) return def;
  return value_to_double(v);
}

static void get_str(const char *buf, size_t len, const char *key, const char *def, char *out, size_t outlen) {
  if (!card_value(buf, len, key, out, outlen)) {
    strncpy(out, def, outlen);
    out[outlen - 1] = '\0';
  }
}

RSG_EXPORT double rawspec_gb300_raw_dms_to_decimal(const char *dms) {
  int sign = 1;
  if (*dms == '-') {
    sign = -1;
    ++dms;
  } else if (*dms == '+') {
    ++dms;
  }
  /* up to three ':'-separated fields: degrees (or hours), minutes, seconds */
  double d = 0.0, scale = 1.0;
  const char *p = dms;
  for (int field = 0; field < 3 && *p; ++field) {
    while (*p == ':') ++p;  /* empty fields are skipped */
    if (!*p) break;
    d += strtod(p, NULL) / scale;
    scale *= 60.0;
    p = strchr(p, ':');
    if (!p) break;
  }
  return sign * d;
}

/* ---------------------------------------------------------------------------
 * Headers
 * ------------------------------------------------------------------------- */

RSG_EXPORT size_t rawspec_gb300_raw_header_size(const char *buf, size_t len, int directio) {
  for (size_t i = 0; i + 4 <= len; i += 80) {
    if (strncmp(buf + i, "END ", 4) == 0) {
      size_t n = i + 80;
      if (directio) n += (RAWSPEC_GB300_RAW_MAX_HDR - n) % 512;  /* to the next 512-byte boundary */
      return n;
    }
  }
  return 0;
}

RSG_EXPORT int rawspec_gb300_raw_parse_header(const char *buf, size_t len, rawspec_gb300_raw_hdr *h) {
  h->blocsize = (size_t)get_s32(buf, len, "BLOCSIZE", 0);
  h->npol = (unsigned)get_s32(buf, len, "NPOL", 0);
  h->obsnchan = (unsigned)get_s32(buf, len, "OBSNCHAN", 0);
  h->nbits = (unsigned)get_ull(buf, len, "NBITS", 8, 0);
  h->obsfreq = get_dbl(buf, len, "OBSFREQ", 0.0);
  h->obsbw = get_dbl(buf, len, "OBSBW", 0.0);
  h->tbin = get_dbl(buf, len, "TBIN", 0.0);
  h->directio = get_s32(buf, len, "DIRECTIO", 0);
  h->pktidx = (int64_t)get_ull(buf, len, "PKTIDX", (unsigned long long)-1, 0);
  h->beam_id = get_s32(buf, len, "BEAM_ID", -1);
  h->nbeam = get_s32(buf, len, "NBEAM", -1);
  h->refbeam = get_s32(buf, len, "REFBEAM", -1);
  h->nants = (unsigned)get_ull(buf, len, "NANTS", 1, 0);
  char tmp[81];
  get_str(buf, len, "RA_STR", "0.0", tmp, sizeof(tmp));
  h->ra = rawspec_gb300_raw_dms_to_decimal(tmp);
  get_str(buf, len, "DEC_STR", "0.0", tmp, sizeof(tmp));
  h->dec = rawspec_gb300_raw_dms_to_decimal(tmp);
  const int imjd = get_s32(buf, len, "STT_IMJD", 51545);
  const int smjd = get_s32(buf, len, "STT_SMJD", 0);
  h->mjd = (double)imjd + (double)smjd / 86400.0;
  get_str(buf, len, "SRC_NAME", "Unknown", h->src_name, 81);
  get_str(buf, len, "TELESCOP", "Unknown", h->telescop, 81);
  return 0;
}

RSG_EXPORT off_t rawspec_gb300_raw_read_header(int fd, rawspec_gb300_raw_hdr *h) {
  static __thread char hdr[RAWSPEC_GB300_RAW_MAX_HDR] __attribute__((aligned(512)));
  const off_t pos = lseek(fd, 0, SEEK_CUR);
  const ssize_t n = read(fd, hdr, sizeof(hdr));
  if (n < 0) return -1;
  if (n < 80) return 0;
  const size_t len = (size_t)n;
  rawspec_gb300_raw_parse_header(hdr, len, h);
  const char *missing = h->blocsize == 0   ? "BLOCSIZE"
                        : h->npol == 0     ? "NPOL"
                        : h->obsnchan == 0 ? "OBSNCHAN"
                        : h->obsfreq == 0.0 ? "OBSFREQ"
                        : h->obsbw == 0.0  ? "OBSBW"
                        : h->tbin == 0.0   ? "TBIN"
                        : h->pktidx == -1  ? "PKTIDX"
                                           : NULL;
  if (missing) {
    fprintf(stderr, "%s not found in header\n", missing);
    return -1;
  }
  if (h->npol == 4) h->npol = 2;  /* four cross products of two polarisations */
  h->hdr_pos = pos;
  h->hdr_size = rawspec_gb300_raw_header_size(hdr, len, 0);
  const size_t skip = rawspec_gb300_raw_header_size(hdr, len, h->directio);
  return lseek(fd, pos + (off_t)skip, SEEK_SET);
}

/* ---------------------------------------------------------------------------
 * Packet-index sequencing
 * ------------------------------------------------------------------------- */

RSG_EXPORT int rawspec_gb300_pktidx_step(rawspec_gb300_pktidx_state *st, int64_t p, int64_t *nfill) {
  *nfill = 0;
  if (!st->started) {  /* the stem's first block sets the reference index */
    st->started = 1;
    st->prev = p;
    st->step = 0;
    return RAWSPEC_GB300_PKT_TAKE;
  }
  if (st->step == 0 && p > st->prev) st->step = p - st->prev;  /* learnt from the first increase */
  const int64_t diff = p - st->prev;
  if (diff != st->step) {
    if (p < st->prev) return RAWSPEC_GB300_PKT_BACKWARD;
    if (diff % st->step != 0) return RAWSPEC_GB300_PKT_MISALIGNED;
    if (diff == 0) return RAWSPEC_GB300_PKT_END_FILE;
    *nfill = diff / st->step - 1;
  }
  st->prev = p;
  return RAWSPEC_GB300_PKT_TAKE;
}

/* ---------------------------------------------------------------------------
 * Streaming
 * ------------------------------------------------------------------------- */

RSG_EXPORT int rawspec_gb300_ingest_geometry(const rawspec_gb300_raw_hdr *h, unsigned int schan, unsigned int nchan,
                                             rawspec_context *ctx, int *expand4) {
  if (h->nants == 0 || h->obsnchan % h->nants != 0) {
    fprintf(stderr, "bad obsnchan/nants: %u %% %u != 0\n", h->obsnchan, h->nants);
    return 1;
  }
  const unsigned Np = h->npol, Nbps = h->nbits;
  const size_t per_sample = (size_t)2 * Np * h->obsnchan * Nbps / 8;  /* bytes per time sample, all channels */
  if (per_sample == 0) return 1;
  const size_t Ntpb = h->blocsize / per_sample;
  if (Ntpb * per_sample != h->blocsize) {
    fprintf(stderr, "bad block geometry: 2*%upol*%uchan*%zutpb*(%ubps/8) != %zu\n", Np, h->obsnchan, Ntpb, Nbps,
            h->blocsize);
    return 1;
  }
  unsigned Nc = h->obsnchan;
  if (nchan != 0) {
    if (schan + nchan > h->obsnchan) {
      fprintf(stderr, "bad channel range: schan + nchan > obsnchan (%u + %u > %u)\n", schan, nchan, h->obsnchan);
      return 1;
    }
    Nc = nchan;
  } else if (schan != 0) {
    fprintf(stderr, "nchan must be non-zero if schan is non-zero\n");
    return 1;
  }
  ctx->Nant = h->nants;
  ctx->Nc = Nc;
  ctx->Np = Np;
  ctx->Ntpb = (unsigned)Ntpb;
  ctx->Nbps = Nbps;
  ctx->input_conjugated = h->obsbw < 0 ? 1 : 0;
  if (expand4) *expand4 = Nbps == 4;
  return 0;
}

/* Reads exactly n bytes (short only at end of file); returns bytes read or -1. */
static ssize_t read_fully(int fd, void *buf, size_t n) {
  size_t got = 0;
  while (got < n) {
    const ssize_t r = read(fd, (char *)buf + got, n - got);
    if (r < 0) {
      if (errno == EINTR) continue;
      return -1;
    }
    if (r == 0) break;
    got += (size_t)r;
  }
  return (ssize_t)got;
}

RSG_EXPORT int rawspec_gb300_ingest_files(rawspec_context *ctx, const char *const *paths, int npaths, unsigned int schan,
                                          int expand4, rawspec_gb300_ingest_stats *st) {
  rawspec_gb300_ingest_stats local;
  if (!st) st = &local;
  memset(st, 0, sizeof(*st));
  if (!ctx || !ctx->h_blkbufs || ctx->Nb == 0 || ctx->Nb_host == 0) return 1;
  /* bytes of one channel of one block in the file and in a host block */
  const size_t file_bits = expand4 ? 4 : ctx->Nbps;
  const size_t chan_bytes = (size_t)2 * ctx->Np * file_bits / 8 * ctx->Ntpb;
  const size_t block_bytes = chan_bytes * ctx->Nc;
  rawspec_gb300_pktidx_state ps;
  memset(&ps, 0, sizeof(ps));
  long long bi = 0;  /* block index across the stem */
  int rc = 0;

  /* hands the host blocks to the GPU when block bi completes a buffer */
#define RSG_BUFFER_DONE()                                                                            \
  do {                                                                                               \
    if (bi % ctx->Nb == ctx->Nb - 1) {                                                               \
      if (rawspec_wait_for_completion(ctx) != 0) return 1;                                           \
      if (rawspec_copy_blocks_to_gpu_and_start_processing(ctx, ctx->Nb, (char)(expand4 ? 1 : 0),    \
                                                          RAWSPEC_FORWARD_FFT) != 0)                 \
        return 1;                                                                                    \
      st->buffers++;                                                                                 \
    }                                                                                                \
  } while (0)

  for (int f = 0; f < npaths && st->stop == 0; ++f) {
    const int fd = open(paths[f], O_RDONLY);
    if (fd < 0) {
      fprintf(stderr, "cannot open %s: %s\n", paths[f], strerror(errno));
      st->stop = -1;
      break;
    }
    rawspec_gb300_raw_hdr h;
    off_t pos = rawspec_gb300_raw_read_header(fd, &h);
    while (pos > 0) {
      if (h.obsnchan < schan + ctx->Nc || chan_bytes * h.obsnchan != h.blocsize) {
        fprintf(stderr, "%s: block geometry differs from the context\n", paths[f]);
        st->stop = -1;
        break;
      }
      int64_t nfill = 0;
      const int act = rawspec_gb300_pktidx_step(&ps, h.pktidx, &nfill);
      if (act == RAWSPEC_GB300_PKT_BACKWARD || act == RAWSPEC_GB300_PKT_MISALIGNED) {
        fprintf(stderr, "%s: %s jump in pktidx to %lld\n", paths[f],
                act == RAWSPEC_GB300_PKT_BACKWARD ? "backwards" : "misaligned", (long long)h.pktidx);
        st->stop = act;
        break;
      }
      if (act == RAWSPEC_GB300_PKT_END_FILE) break;  /* the rest of this file is skipped */
      for (int64_t z = 0; z < nfill; ++z) {  /* missing blocks: zeros */
        memset(ctx->h_blkbufs[bi % ctx->Nb_host], 0, block_bytes);
        st->blocks_zero++;
        RSG_BUFFER_DONE();
        ++bi;
      }
      /* the block's channels [schan, schan + Nc) */
      if (lseek(fd, (off_t)(chan_bytes * schan), SEEK_CUR) < 0) {
        st->stop = -1;
        break;
      }
      const ssize_t got = read_fully(fd, ctx->h_blkbufs[bi % ctx->Nb_host], block_bytes);
      if (got < 0 || (size_t)got < block_bytes) {
        fprintf(stderr, "%s: %s\n", paths[f], got < 0 ? strerror(errno) : "incomplete block at end of file");
        st->stop = -1;
        break;
      }
      lseek(fd, (off_t)(chan_bytes * (h.obsnchan - schan - ctx->Nc)), SEEK_CUR);
      st->blocks_read++;
      RSG_BUFFER_DONE();
      ++bi;
      pos = rawspec_gb300_raw_read_header(fd, &h);
    }
    if (pos < 0) fprintf(stderr, "%s: cannot read a block header\n", paths[f]);
    close(fd);
  }
#undef RSG_BUFFER_DONE
  if (rawspec_wait_for_completion(ctx) != 0) rc = 1;
  return rc;
}
