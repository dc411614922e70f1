/* io_fil.c -- SIGPROC filterbank output of the spectrometer's dumps.
 *
 * The header format (length-prefixed keyword strings followed by
 * little-endian int32 / float64 values, angles as ddmmss.s) and the keyword
 * order are those the reference writes (rawspec_fbutils.c:246-322), so that
 * its readers and downstream tools see the same files; the per-product
 * header values follow the reference CLI (rawspec.c:484-492, 800-826) and
 * the write order of the dumps its file callback (rawspec_file.c:102-243).
 * The code is this project's own. */
#define _GNU_SOURCE
#include <errno.h>
#include <fcntl.h>
#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <strings.h>
#include <sys/stat.h>
#include <unistd.h>

#include "rawspec_gb300_io.h"

#define RSG_EXPORT __attribute__((visibility("default")))

/* ---------------------------------------------------------------------------
 * Header serialisation
 * ------------------------------------------------------------------------- */

typedef struct {
  unsigned char *p, *end;
  int overflow;
} Sink;

static void put_bytes(Sink *s, const void *src, size_t n) {
  if (s->overflow || (size_t)(s->end - s->p) < n) {
    s->overflow = 1;
    return;
  }
  memcpy(s->p, src, n);
  s->p += n;
}

static void put_i32(Sink *s, int32_t v) {
  const uint32_t u = (uint32_t)v;
  const unsigned char b[4] = {(unsigned char)u, (unsigned char)(u >> 8), (unsigned char)(u >> 16),
                              (unsigned char)(u >> 24)};
  put_bytes(s, b, 4);
}

static void put_f64(Sink *s, double d) {
  uint64_t u;
  memcpy(&u, &d, 8);
  unsigned char b[8];
  for (int i = 0; i < 8; ++i) b[i] = (unsigned char)(u >> (8 * i));
  put_bytes(s, b, 8);
}

/* a string: int32 length (at most 80 characters are written) and the bytes */
static void put_str(Sink *s, const char *c) {
  const size_t n = strnlen(c, 80);
  put_i32(s, (int32_t)n);
  put_bytes(s, c, n);
}

/* decimal degrees (or hours) -> sign * ddmmss.s */
static double to_dms(double x) {
  const int sign = x < 0 ? -1 : 1;
  x = fabs(x);
  const double m = 60.0 * fmod(x, 1.0);
  const double sec = 60.0 * fmod(m, 1.0);
  return sign * (10000.0 * floor(x) + 100.0 * floor(m) + sec);
}

RSG_EXPORT long rawspec_gb300_fil_header(const rawspec_gb300_fil_hdr *h, void *buf, size_t cap) {
  return rawspec_gb300_fil_header_padded(h, buf, cap, 0);
}

/* The header, padded to at least minlen bytes by extra "rawdatafile" entries
 * of blanks placed before the real one (the later entry wins in a reader):
 * whole 79-byte entries while more than 98 bytes are missing, then one entry
 * of the remaining length if it exceeds 19 bytes (rawspec_fbutils.c:330-404). */
RSG_EXPORT long rawspec_gb300_fil_header_padded(const rawspec_gb300_fil_hdr *h, void *buf, size_t cap,
                                                int minlen) {
  Sink s = {(unsigned char *)buf, (unsigned char *)buf + cap, 0};
  put_str(&s, "HEADER_START");
  put_str(&s, "machine_id");
  put_i32(&s, h->machine_id);
  put_str(&s, "telescope_id");
  put_i32(&s, h->telescope_id);
  put_str(&s, "src_raj");
  put_f64(&s, to_dms(h->src_raj));
  put_str(&s, "src_dej");
  put_f64(&s, to_dms(h->src_dej));
  put_str(&s, "az_start");
  put_f64(&s, h->az_start);
  put_str(&s, "za_start");
  put_f64(&s, h->za_start);
  put_str(&s, "data_type");
  put_i32(&s, h->data_type);
  put_str(&s, "fch1");
  put_f64(&s, h->fch1);
  put_str(&s, "foff");
  put_f64(&s, h->foff);
  put_str(&s, "nchans");
  put_i32(&s, h->nchans);
  put_str(&s, "nbeams");
  put_i32(&s, h->nbeams);
  put_str(&s, "ibeam");
  put_i32(&s, h->ibeam);
  put_str(&s, "nbits");
  put_i32(&s, h->nbits);
  put_str(&s, "tstart");
  put_f64(&s, h->tstart);
  put_str(&s, "tsamp");
  put_f64(&s, h->tsamp);
  put_str(&s, "nifs");
  put_i32(&s, h->nifs);
  if (h->barycentric) {  /* optional flags, only when set */
    put_str(&s, "barycentric");
    put_i32(&s, h->barycentric);
  }
  if (h->pulsarcentric) {
    put_str(&s, "pulsarcentric");
    put_i32(&s, h->pulsarcentric);
  }
  put_str(&s, "source_name");
  put_str(&s, h->source_name);
  /* bytes still missing once the rawdatafile entry and HEADER_END are added */
  long pad = (long)minlen - (long)(s.p - (unsigned char *)buf) - (8 + 11 + (long)strnlen(h->rawdatafile, 80)) -
             (4 + 10);
  char blanks[80];
  memset(blanks, ' ', sizeof(blanks) - 1);
  blanks[sizeof(blanks) - 1] = '\0';
  while (pad > 98) {
    blanks[60] = '\0';  /* 4 + 11 + 4 + 60 = 79 bytes */
    put_str(&s, "rawdatafile");
    put_str(&s, blanks);
    pad -= 79;
  }
  if (pad > 19) {
    blanks[60] = ' ';
    blanks[pad - 19] = '\0';
    put_str(&s, "rawdatafile");
    put_str(&s, blanks);
  }
  put_str(&s, "rawdatafile");
  put_str(&s, h->rawdatafile);
  put_str(&s, "HEADER_END");
  return s.overflow ? -1 : (long)(s.p - (unsigned char *)buf);
}

RSG_EXPORT int rawspec_gb300_telescope_id(const char *name) {
  /* SIGPROC telescope identifiers */
  static const struct {
    const char *name;
    int id;
  } ids[] = {{"FAKE", 0},     {"ARECIBO", 1}, {"OOTY", 2},        {"NANCAY", 3}, {"PARKES", 4},
             {"JODRELL", 5},  {"GBT", 6},     {"GMRT", 7},        {"EFFELSBERG", 8}, {"140FT", 9},
             {"ATA", 9},      {"SRT", 10},    {"LEUSCHNER", 11},  {"MEERKAT", 64}};
  for (size_t i = 0; i < sizeof(ids) / sizeof(ids[0]); ++i)
    if (strcasecmp(name, ids[i].name) == 0) return ids[i].id;
  return -1;
}

RSG_EXPORT int rawspec_gb300_fil_header_for_product(const rawspec_gb300_raw_hdr *raw, const rawspec_context *ctx,
                                                    int product, unsigned int schan, const char *rawdatafile,
                                                    rawspec_gb300_fil_hdr *h) {
  if (!raw || !ctx || !h || product < 0 || product >= (int)ctx->No || raw->nants == 0) return 1;
  memset(h, 0, sizeof(*h));
  const double Nt = (double)ctx->Nts[product];
  const double ncpa = (double)(raw->obsnchan / raw->nants);  /* coarse channels per antenna */
  h->machine_id = 20;
  h->data_type = 1;
  h->nbeams = 1;
  h->nbits = 32;
  h->nifs = abs(ctx->Npolout[product]);
  h->telescope_id = rawspec_gb300_telescope_id(raw->telescop);
  h->src_raj = raw->ra;
  h->src_dej = raw->dec;
  h->tstart = raw->mjd;
  h->ibeam = raw->beam_id;
  h->refbeam = raw->refbeam;
  snprintf(h->source_name, sizeof(h->source_name), "%s", raw->src_name);
  snprintf(h->rawdatafile, sizeof(h->rawdatafile), "%s", rawdatafile ? rawdatafile : "");
  /* OBSBW is one antenna's bandwidth; OBSNCHAN counts all antennas' channels */
  h->foff = raw->obsbw / ncpa / Nt;
  h->fch1 = raw->obsfreq - raw->obsbw * (ncpa - 1) / (2 * ncpa) - (double)(ctx->Nts[product] / 2) * h->foff +
            (double)(schan % (raw->obsnchan / raw->nants)) * raw->obsbw / ncpa;
  h->nfpc = (int)ctx->Nts[product];
  h->nchans = (int)(ctx->Nc * ctx->Nts[product] / raw->nants);
  h->tsamp = raw->tbin * Nt * (double)ctx->Nas[product];
  return 0;
}

/* ---------------------------------------------------------------------------
 * File writer
 * ------------------------------------------------------------------------- */

struct rawspec_gb300_fil_writer {
  int nfd;            /* product files: 1, or one per antenna */
  int fd[RAWSPEC_GB300_MAX_FIL_FILES];
  int fd_ics;         /* -1 if none */
  int per_antenna;
  unsigned Nant, Nds, nifs;
  const float *pwr;   /* host dump buffers of the product */
  const float *ics;
  size_t pwr_bytes;
  pthread_t thread;
  int thread_valid;
  int failed;
};

static int open_fil(const char *dest, const char *stem, int idx, char *path, size_t cap) {
  if (dest && dest[0]) {
    const char *base = strrchr(stem, '/');
    base = base ? base + 1 : stem;
    snprintf(path, cap, "%s/%s.rawspec.%04d.fil", dest, base, idx);
  } else {
    snprintf(path, cap, "%s.rawspec.%04d.fil", stem, idx);
  }
  return open(path, O_WRONLY | O_CREAT | O_TRUNC, 0664);
}

static int write_all(int fd, const void *p, size_t n) {
  const char *c = (const char *)p;
  while (n) {
    const ssize_t w = write(fd, c, n);
    if (w < 0) {
      if (errno == EINTR) continue;
      return -1;
    }
    c += w;
    n -= (size_t)w;
  }
  return 0;
}

static int write_header(int fd, const rawspec_gb300_fil_hdr *h) {
  unsigned char buf[4096];
  const long n = rawspec_gb300_fil_header(h, buf, sizeof(buf));
  return n < 0 ? -1 : write_all(fd, buf, (size_t)n);
}

RSG_EXPORT rawspec_gb300_fil_writer *rawspec_gb300_fil_writer_open(const rawspec_context *ctx, int product,
                                                                   const rawspec_gb300_fil_hdr *hdr, const char *dest,
                                                                   const char *stem, int output_idx, int per_antenna,
                                                                   const char *ics_stem) {
  if (!ctx || !hdr || !stem || product < 0 || product >= (int)ctx->No) return NULL;
  const unsigned Nant = ctx->Nant ? ctx->Nant : 1;
  /* several antennas are written one file each unless only their sum is wanted */
  const int split = Nant > 1 && (per_antenna || !ctx->incoherently_sum);
  if (split && Nant > RAWSPEC_GB300_MAX_FIL_FILES) return NULL;
  rawspec_gb300_fil_writer *w = (rawspec_gb300_fil_writer *)calloc(1, sizeof(*w));
  if (!w) return NULL;
  w->per_antenna = split;
  w->Nant = Nant;
  w->Nds = ctx->Nds[product];
  w->nifs = (unsigned)abs(ctx->Npolout[product]);
  w->pwr = ctx->h_pwrbuf[product];
  w->ics = ctx->incoherently_sum ? ctx->h_icsbuf[product] : NULL;
  w->pwr_bytes = ctx->h_pwrbuf_size[product];
  w->fd_ics = -1;
  char path[PATH_MAX + 1], ant_stem[PATH_MAX + 1];
  /* product files: one file (a single antenna, or all antennas together, which
   * only the incoherent sum writes), or one per antenna */
  w->nfd = split ? (int)Nant : 1;
  for (int a = 0; a < w->nfd; ++a) {
    if (split)
      snprintf(ant_stem, sizeof(ant_stem), "%s-ant%03d", stem, a);
    else
      snprintf(ant_stem, sizeof(ant_stem), "%s", stem);
    w->fd[a] = -1;
    if (!split && Nant > 1 && w->ics) continue;  /* summed antennas: only the sum is written */
    w->fd[a] = open_fil(dest, ant_stem, output_idx, path, sizeof(path));
    if (w->fd[a] < 0 || write_header(w->fd[a], hdr) != 0) {
      fprintf(stderr, "cannot open output file %s: %s\n", path, strerror(errno));
      rawspec_gb300_fil_writer_close(w);
      return NULL;
    }
  }
  if (w->ics) {
    w->fd_ics = open_fil(dest, ics_stem ? ics_stem : stem, output_idx, path, sizeof(path));
    if (w->fd_ics < 0 || write_header(w->fd_ics, hdr) != 0) {
      fprintf(stderr, "cannot open output file %s: %s\n", path, strerror(errno));
      rawspec_gb300_fil_writer_close(w);
      return NULL;
    }
  }
  return w;
}

/* Writes one dump of the product (run on the writer thread). */
static void *write_dump(void *arg) {
  rawspec_gb300_fil_writer *w = (rawspec_gb300_fil_writer *)arg;
  if (w->Nant == 1 && w->fd[0] >= 0) {
    if (write_all(w->fd[0], w->pwr, w->pwr_bytes)) w->failed = 1;
  } else if (w->per_antenna) {
    /* [Nds][nifs][Nant][Nc/Nant][Nt]: per spectrum and polarisation, each
     * antenna's channels to its own file */
    const size_t spectrum = w->pwr_bytes / sizeof(float) / w->Nds;
    const size_t plane = spectrum / w->nifs;
    const size_t ant = plane / w->Nant;
    for (size_t k = 0; k < w->Nds && !w->failed; ++k)
      for (size_t j = 0; j < w->nifs && !w->failed; ++j)
        for (size_t i = 0; i < w->Nant; ++i)
          if (write_all(w->fd[i], w->pwr + k * spectrum + j * plane + i * ant, ant * sizeof(float))) {
            w->failed = 1;
            break;
          }
  }
  if (w->fd_ics >= 0 && w->ics && !w->failed)
    if (write_all(w->fd_ics, w->ics, w->pwr_bytes / w->Nant)) w->failed = 1;
  return NULL;
}

static void join_writer(rawspec_gb300_fil_writer *w) {
  if (w->thread_valid) {
    pthread_join(w->thread, NULL);
    w->thread_valid = 0;
  }
}

RSG_EXPORT int rawspec_gb300_fil_writer_close(rawspec_gb300_fil_writer *w) {
  if (!w) return 0;
  join_writer(w);
  int bad = w->failed;
  for (int a = 0; a < w->nfd; ++a)
    if (w->fd[a] >= 0 && close(w->fd[a]) != 0) bad = 1;
  if (w->fd_ics >= 0 && close(w->fd_ics) != 0) bad = 1;
  free(w);
  return bad ? 1 : 0;
}

RSG_EXPORT void rawspec_gb300_fil_dump_callback(rawspec_context *ctx, int output_product, int callback_type) {
  rawspec_gb300_fil_writer **ws = (rawspec_gb300_fil_writer **)ctx->user_data;
  if (!ws || !ws[output_product]) return;
  rawspec_gb300_fil_writer *w = ws[output_product];
  if (callback_type == RAWSPEC_CALLBACK_PRE_DUMP) {
    join_writer(w);  /* the host buffers are about to be overwritten */
  } else if (callback_type == RAWSPEC_CALLBACK_POST_DUMP) {
    join_writer(w);
    if (pthread_create(&w->thread, NULL, write_dump, w) == 0)
      w->thread_valid = 1;
    else
      write_dump(w);
  }
  if (w->failed) ctx->exit_soon = 1;
}
