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
#include <pthread.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <unistd.h>

#include <cuda_runtime_api.h>

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

/* ---------------------------------------------------------------------------
 * Block reads: a block's channel range is one contiguous byte range of the
 * file, read (or zero-filled) by a small pool of threads in 4 KiB-aligned
 * stripes with pread, so that the page-cache copies are not limited to one
 * core.  RAWSPEC_GB300_INGEST_THREADS sets the pool size (default: the
 * online CPUs, at most 16).
 * ------------------------------------------------------------------------- */
#define RSG_MAX_READERS 16

typedef struct {
  int nthreads;  /* readers taking part, the calling thread included */
  int quit;
  pthread_barrier_t start, done;
  pthread_mutex_t gate_mu;
  pthread_cond_t gate_cv;
  int gate;      /* set once the barriers are sized for the readers that started */
  pthread_t tid[RSG_MAX_READERS];
  /* the current job */
  int fd;
  off_t off;
  char *dst;
  size_t bytes;
  int zero;
  size_t want[RSG_MAX_READERS], got[RSG_MAX_READERS];
} ReaderPool;

typedef struct {
  ReaderPool *pool;
  int k;
} ReaderArg;

static void do_stripe(ReaderPool *p, int k) {
  const size_t a = (p->bytes * (size_t)k / (size_t)p->nthreads) & ~(size_t)4095;
  const size_t b = k + 1 == p->nthreads ? p->bytes : (p->bytes * (size_t)(k + 1) / (size_t)p->nthreads) & ~(size_t)4095;
  const size_t n = b > a ? b - a : 0;
  size_t got = 0;
  if (p->zero) {
    memset(p->dst + a, 0, n);
    got = n;
  } else {
    while (got < n) {
      const ssize_t r = pread(p->fd, p->dst + a + got, n - got, p->off + (off_t)(a + got));
      if (r < 0) {
        if (errno == EINTR) continue;
        break;
      }
      if (r == 0) break;
      got += (size_t)r;
    }
  }
  p->want[k] = n;
  p->got[k] = got;
}

static void *reader_main(void *arg) {
  ReaderArg *ra = (ReaderArg *)arg;
  ReaderPool *p = ra->pool;
  pthread_mutex_lock(&p->gate_mu);
  while (!p->gate) pthread_cond_wait(&p->gate_cv, &p->gate_mu);
  pthread_mutex_unlock(&p->gate_mu);
  for (;;) {
    pthread_barrier_wait(&p->start);
    if (p->quit) break;
    do_stripe(p, ra->k);
    pthread_barrier_wait(&p->done);
  }
  return NULL;
}

static void pool_start(ReaderPool *p, ReaderArg *args) {
  memset(p, 0, sizeof(*p));
  long n = sysconf(_SC_NPROCESSORS_ONLN);
  const char *env = getenv("RAWSPEC_GB300_INGEST_THREADS");
  if (env && atoi(env) > 0) n = atoi(env);
  if (n < 1) n = 1;
  if (n > RSG_MAX_READERS) n = RSG_MAX_READERS;
  pthread_mutex_init(&p->gate_mu, NULL);
  pthread_cond_init(&p->gate_cv, NULL);
  /* start the readers; they wait at the gate until the barriers exist */
  int started = 1;
  for (int k = 1; k < n; ++k) {
    args[k].pool = p;
    args[k].k = k;
    if (pthread_create(&p->tid[k], NULL, reader_main, &args[k]) != 0) break;
    ++started;
  }
  p->nthreads = started;
  if (started > 1) {
    pthread_barrier_init(&p->start, NULL, (unsigned)started);
    pthread_barrier_init(&p->done, NULL, (unsigned)started);
  }
  pthread_mutex_lock(&p->gate_mu);
  p->gate = 1;
  pthread_cond_broadcast(&p->gate_cv);
  pthread_mutex_unlock(&p->gate_mu);
}

static void pool_stop(ReaderPool *p) {
  if (p->nthreads > 1) {
    p->quit = 1;
    pthread_barrier_wait(&p->start);
    for (int k = 1; k < p->nthreads; ++k) pthread_join(p->tid[k], NULL);
    pthread_barrier_destroy(&p->start);
    pthread_barrier_destroy(&p->done);
  }
  pthread_cond_destroy(&p->gate_cv);
  pthread_mutex_destroy(&p->gate_mu);
}

/* Reads `bytes` at file offset `off` into dst (or zero-fills dst when fd < 0);
 * returns 0 if every byte was read. */
static int pool_read(ReaderPool *p, int fd, off_t off, char *dst, size_t bytes) {
  p->fd = fd;
  p->off = off;
  p->dst = dst;
  p->bytes = bytes;
  p->zero = fd < 0;
  if (p->nthreads > 1) pthread_barrier_wait(&p->start);
  do_stripe(p, 0);
  if (p->nthreads > 1) pthread_barrier_wait(&p->done);
  for (int k = 0; k < p->nthreads; ++k)
    if (p->got[k] != p->want[k]) return 1;
  return 0;
}

/* ---------------------------------------------------------------------------
 * The stem's blocks are read on a reader thread into one of two sets of
 * pinned host blocks while the calling thread hands the other set to the GPU
 * (wait_for_completion + copy_blocks_to_gpu_and_start_processing, with the
 * context's block pointers switched to that set), so that file reads
 * overlap the host-to-device copies.  The context's own blocks are the first
 * set and are restored at the end; the second set is allocated here.  Only
 * the calling thread calls the library.
 * ------------------------------------------------------------------------- */
#define RSG_MAX_NB 64

typedef struct {
  /* fixed */
  rawspec_context *ctx;
  const char *const *paths;
  int npaths;
  unsigned schan;
  size_t chan_bytes, block_bytes;
  char *sets[2][RSG_MAX_NB];
  ReaderPool *pool;
  /* hand-off */
  pthread_mutex_t mu;
  pthread_cond_t cv;
  int filled[2];   /* a full buffer waits in the set */
  int busy[2];     /* the set is being filled or handed over */
  int reader_done;
  int abort;
  /* results (reader) */
  long long blocks_read, blocks_zero;
  int stop;
} Ingest;

/* Reader: claims set k (waits while the GPU side still uses it). */
static int claim_set(Ingest *in, int k) {
  pthread_mutex_lock(&in->mu);
  while ((in->filled[k] || in->busy[k]) && !in->abort) pthread_cond_wait(&in->cv, &in->mu);
  const int ok = !in->abort;
  if (ok) in->busy[k] = 1;
  pthread_mutex_unlock(&in->mu);
  return ok;
}

static void publish_set(Ingest *in, int k) {
  pthread_mutex_lock(&in->mu);
  in->busy[k] = 0;
  in->filled[k] = 1;
  pthread_cond_broadcast(&in->cv);
  pthread_mutex_unlock(&in->mu);
}

static void *ingest_reader(void *arg) {
  Ingest *in = (Ingest *)arg;
  rawspec_context *ctx = in->ctx;
  rawspec_gb300_pktidx_state ps;
  memset(&ps, 0, sizeof(ps));
  long long bi = 0;  /* block index across the stem */
  int set = 0;
  int have = claim_set(in, 0);
  for (int f = 0; f < in->npaths && in->stop == 0 && have; ++f) {
    const int fd = open(in->paths[f], O_RDONLY);
    if (fd < 0) {
      fprintf(stderr, "cannot open %s: %s\n", in->paths[f], strerror(errno));
      in->stop = -1;
      break;
    }
    rawspec_gb300_raw_hdr h;
    off_t pos = rawspec_gb300_raw_read_header(fd, &h);
    while (pos > 0 && have) {
      if (h.obsnchan < in->schan + ctx->Nc || in->chan_bytes * h.obsnchan != h.blocsize) {
        fprintf(stderr, "%s: block geometry differs from the context\n", in->paths[f]);
        in->stop = -1;
        break;
      }
      int64_t nfill = 0;
      const int act = rawspec_gb300_pktidx_step(&ps, h.pktidx, &nfill);
      if (act == RAWSPEC_GB300_PKT_BACKWARD || act == RAWSPEC_GB300_PKT_MISALIGNED) {
        fprintf(stderr, "%s: %s jump in pktidx to %lld\n", in->paths[f],
                act == RAWSPEC_GB300_PKT_BACKWARD ? "backwards" : "misaligned", (long long)h.pktidx);
        in->stop = act;
        break;
      }
      if (act == RAWSPEC_GB300_PKT_END_FILE) break;  /* the rest of this file is skipped */
      /* missing blocks (zeros), then the block's channels [schan, schan + Nc) */
      for (int64_t z = 0; z <= nfill && have; ++z) {
        char *dst = in->sets[set][bi % ctx->Nb];
        if (z < nfill) {
          pool_read(in->pool, -1, 0, dst, in->block_bytes);
          in->blocks_zero++;
        } else {
          if (pool_read(in->pool, fd, pos + (off_t)(in->chan_bytes * in->schan), dst, in->block_bytes) != 0) {
            fprintf(stderr, "%s: incomplete block at end of file\n", in->paths[f]);
            in->stop = -1;
            break;
          }
          in->blocks_read++;
        }
        if (bi % ctx->Nb == ctx->Nb - 1) {  /* a full buffer: hand it over, go on in the other set */
          publish_set(in, set);
          set ^= 1;
          have = claim_set(in, set);
        }
        ++bi;
      }
      if (in->stop) break;
      if (lseek(fd, pos + (off_t)h.blocsize, SEEK_SET) < 0) {
        in->stop = -1;
        break;
      }
      pos = rawspec_gb300_raw_read_header(fd, &h);
    }
    if (pos < 0) fprintf(stderr, "%s: cannot read a block header\n", in->paths[f]);
    close(fd);
  }
  pthread_mutex_lock(&in->mu);
  if (have) in->busy[set] = 0;  /* a partial buffer is dropped */
  in->reader_done = 1;
  pthread_cond_broadcast(&in->cv);
  pthread_mutex_unlock(&in->mu);
  return NULL;
}

/* The reusable part of an ingest: the second set of host blocks and the
 * reader pool. */
struct rawspec_gb300_ingest {
  rawspec_context *ctx;
  int expand4;
  size_t chan_bytes, block_bytes;
  char *second[RSG_MAX_NB];
  ReaderPool pool;
  ReaderArg args[RSG_MAX_READERS];
};

RSG_EXPORT rawspec_gb300_ingest *rawspec_gb300_ingest_open(rawspec_context *ctx, int expand4) {
  if (!ctx || !ctx->h_blkbufs || ctx->Nb == 0 || ctx->Nb > RSG_MAX_NB || ctx->Nb_host < ctx->Nb) return NULL;
  rawspec_gb300_ingest *g = (rawspec_gb300_ingest *)calloc(1, sizeof(*g));
  if (!g) return NULL;
  g->ctx = ctx;
  g->expand4 = expand4;
  /* bytes of one channel of one block in the file and in a host block */
  const size_t file_bits = expand4 ? 4 : ctx->Nbps;
  g->chan_bytes = (size_t)2 * ctx->Np * file_bits / 8 * ctx->Ntpb;
  g->block_bytes = g->chan_bytes * ctx->Nc;
  for (unsigned b = 0; b < ctx->Nb; ++b)
    if (cudaHostAlloc((void **)&g->second[b], g->block_bytes, cudaHostAllocPortable) != cudaSuccess) {
      for (unsigned i = 0; i < b; ++i) cudaFreeHost(g->second[i]);
      free(g);
      return NULL;
    }
  pool_start(&g->pool, g->args);
  return g;
}

RSG_EXPORT void rawspec_gb300_ingest_close(rawspec_gb300_ingest *g) {
  if (!g) return;
  pool_stop(&g->pool);
  for (unsigned b = 0; b < g->ctx->Nb; ++b) cudaFreeHost(g->second[b]);
  free(g);
}

RSG_EXPORT int rawspec_gb300_ingest_stem(rawspec_gb300_ingest *g, const char *const *paths, int npaths,
                                         unsigned int schan, rawspec_gb300_ingest_stats *st) {
  rawspec_gb300_ingest_stats local;
  if (!st) st = &local;
  memset(st, 0, sizeof(*st));
  if (!g) return 1;
  rawspec_context *ctx = g->ctx;
  Ingest in;
  memset(&in, 0, sizeof(in));
  in.ctx = ctx;
  in.paths = paths;
  in.npaths = npaths;
  in.schan = schan;
  in.chan_bytes = g->chan_bytes;
  in.block_bytes = g->block_bytes;
  in.pool = &g->pool;
  char *own[RSG_MAX_NB];
  for (unsigned b = 0; b < ctx->Nb; ++b) {
    own[b] = ctx->h_blkbufs[b];
    in.sets[0][b] = own[b];
    in.sets[1][b] = g->second[b];
  }
  int lib_error = 0;
  pthread_mutex_init(&in.mu, NULL);
  pthread_cond_init(&in.cv, NULL);
  pthread_t reader;
  if (pthread_create(&reader, NULL, ingest_reader, &in) != 0) {
    fprintf(stderr, "rawspec_gb300_ingest_stem: cannot start the reader thread\n");
    pthread_cond_destroy(&in.cv);
    pthread_mutex_destroy(&in.mu);
    return 1;
  }
  /* GPU side: hand over the filled sets in turn */
  int k = 0;
  for (;;) {
    pthread_mutex_lock(&in.mu);
    while (!in.filled[k] && !in.reader_done) pthread_cond_wait(&in.cv, &in.mu);
    const int ready = in.filled[k];
    pthread_mutex_unlock(&in.mu);
    if (!ready) break;
    for (unsigned b = 0; b < ctx->Nb; ++b) ctx->h_blkbufs[b] = in.sets[k][b];
    if (rawspec_wait_for_completion(ctx) != 0 ||
        rawspec_copy_blocks_to_gpu_and_start_processing(ctx, ctx->Nb, (char)(g->expand4 ? 1 : 0),
                                                        RAWSPEC_FORWARD_FFT) != 0)
      lib_error = 1;
    else
      st->buffers++;
    pthread_mutex_lock(&in.mu);
    in.filled[k] = 0;  /* the copy is done: the set may be refilled */
    if (lib_error) in.abort = 1;
    pthread_cond_broadcast(&in.cv);
    pthread_mutex_unlock(&in.mu);
    if (lib_error) break;
    k ^= 1;
  }
  pthread_join(reader, NULL);
  if (rawspec_wait_for_completion(ctx) != 0) lib_error = 1;
  for (unsigned b = 0; b < ctx->Nb; ++b) ctx->h_blkbufs[b] = own[b];
  pthread_cond_destroy(&in.cv);
  pthread_mutex_destroy(&in.mu);
  st->blocks_read = in.blocks_read;
  st->blocks_zero = in.blocks_zero;
  st->stop = in.stop;
  return lib_error ? 1 : 0;
}

RSG_EXPORT int rawspec_gb300_ingest_files(rawspec_context *ctx, const char *const *paths, int npaths, unsigned int schan,
                                          int expand4, rawspec_gb300_ingest_stats *st) {
  rawspec_gb300_ingest *g = rawspec_gb300_ingest_open(ctx, expand4);
  if (!g) {
    if (st) memset(st, 0, sizeof(*st));
    return 1;
  }
  const int rc = rawspec_gb300_ingest_stem(g, paths, npaths, schan, st);
  rawspec_gb300_ingest_close(g);
  return rc;
}
