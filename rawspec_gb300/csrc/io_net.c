/* io_net.c -- UDP output of the spectrometer's dumps.
 *
 * Behaviour of the reference's network output (rawspec_socket.c:21-354, the
 * rate split of rawspec.c:884-901): a connected IPv4 UDP socket; each dump of
 * a product is cut into packets of at most 2048 floats, every packet led by
 * a SIGPROC header describing just that packet (its channel count, first
 * channel frequency and start time) and padded so that the floats start on a
 * 512-byte boundary of a packet-socket capture frame, whose UDP payload
 * begins 0x6c bytes into the frame; the sender paces itself to the product's
 * share of the requested rate.  The packet layout is a wire format receivers
 * depend on, so it is kept alike; the code is this project's own. */
#define _GNU_SOURCE
#include <errno.h>
#include <netdb.h>
#include <netinet/in.h>
#include <pthread.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <sys/socket.h>
#include <sys/types.h>
#include <time.h>
#include <unistd.h>

#include "rawspec_gb300_io.h"

#define RSG_EXPORT __attribute__((visibility("default")))

enum {
  kMinMtu = 8600,
  kMaxFloats = 8192 / (int)sizeof(float),  /* data floats per packet */
  kFrameOffset = 0x6c,                     /* UDP payload offset in a packet-socket frame */
  kPacketBytes = 90000
};

RSG_EXPORT int rawspec_gb300_net_open(const char *host, const char *port) {
  struct addrinfo hints, *res = NULL, *rp;
  memset(&hints, 0, sizeof(hints));
  hints.ai_family = AF_INET;
  hints.ai_socktype = SOCK_DGRAM;
  const int rc = getaddrinfo(host, port, &hints, &res);
  if (rc != 0) {
    fprintf(stderr, "getaddrinfo: %s\n", gai_strerror(rc));
    return -1;
  }
  int fd = -1;
  for (rp = res; rp; rp = rp->ai_next) {
    fd = socket(rp->ai_family, rp->ai_socktype, rp->ai_protocol);
    if (fd < 0) continue;
    if (connect(fd, rp->ai_addr, rp->ai_addrlen) == 0) break;
    close(fd);
    fd = -1;
  }
  freeaddrinfo(res);
  if (fd < 0) {
    fprintf(stderr, "could not open output socket\n");
    return -1;
  }
  int mtu = 0;
  socklen_t len = sizeof(mtu);
  if (getsockopt(fd, IPPROTO_IP, IP_MTU, &mtu, &len) < 0) {
    perror("getsockopt");
    fprintf(stderr, "warning: could not determine MTU\n");
  } else if (mtu < kMinMtu) {
    fprintf(stderr, "MTU %d is too small, need at least %d\n", mtu, kMinMtu);
    close(fd);
    return -1;
  }
  int probe = IP_PMTUDISC_PROBE;  /* set DF, ignore path-MTU changes */
  if (setsockopt(fd, IPPROTO_IP, IP_MTU_DISCOVER, &probe, sizeof(probe)) < 0)
    fprintf(stderr, "warning: could not set IP_MTU_DISCOVER to IP_PMTUDISC_PROBE\n");
  return fd;
}

RSG_EXPORT void rawspec_gb300_net_rates(const rawspec_context *ctx, double total_gbps, double *rates_gbps) {
  double sum_inv = 0.0;
  for (unsigned i = 0; i < ctx->No; i++) sum_inv += 1.0 / ctx->Nas[i];
  for (unsigned i = 0; i < ctx->No; i++) rates_gbps[i] = total_gbps / ctx->Nas[i] / sum_inv;
}

struct rawspec_gb300_net_writer {
  const rawspec_context *ctx;
  int product;
  rawspec_gb300_fil_hdr hdr;  /* per-dump template; tstart advances from dump to dump */
  int fd;
  double rate;                /* Gbit/s: 8 bytes per ns at 64 */
  unsigned char *pkt;
  pthread_t thread;
  int thread_valid;
  rawspec_gb300_net_stats st;
};

static int64_t ns_between(const struct timespec *a, const struct timespec *b) {
  return (int64_t)(b->tv_sec - a->tv_sec) * 1000000000LL + (b->tv_nsec - a->tv_nsec);
}

static void sleep_ns(int64_t ns) {
  if (ns <= 0) return;
  struct timespec t = {(time_t)(ns / 1000000000LL), (long)(ns % 1000000000LL)};
  nanosleep(&t, NULL);
}

static void *net_send(void *arg) {
  rawspec_gb300_net_writer *w = (rawspec_gb300_net_writer *)arg;
  const rawspec_context *ctx = w->ctx;
  rawspec_gb300_fil_hdr *h = &w->hdr;
  const int nchans = h->nchans;
  const double fch1 = h->fch1;
  const unsigned nds = ctx->Nds[w->product];
  const float *pwr = ctx->h_pwrbuf[w->product];
  int cpp, spp;  /* channels and spectra per packet */
  if (nchans >= kMaxFloats) {
    cpp = kMaxFloats;
    spp = 1;
  } else {
    cpp = nchans;
    spp = kMaxFloats / nchans;
    if (spp > (int)nds) spp = (int)nds;
  }
  long long packets = 0, bytes = 0, errors = 0;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  unsigned spec_left = nds;
  while (spec_left) {
    const int nspec = (int)spec_left < spp ? (int)spec_left : spp;
    h->fch1 = fch1;
    const float *src = pwr + (size_t)(nds - spec_left) * nchans;
    int chan_left = nchans;
    while (chan_left) {
      const int nchan = chan_left < cpp ? chan_left : cpp;
      h->nchans = nchan;
      long hl = rawspec_gb300_fil_header(h, w->pkt, kPacketBytes);
      /* data at the next 512-byte boundary of the capture frame; a gap of
       * fewer than 20 bytes cannot hold a padding entry: one block more */
      long off = kFrameOffset + hl;
      if (off % 512) off += 512 - off % 512;
      if (off > kFrameOffset + hl) {
        if (off < kFrameOffset + hl + 20) off += 512;
        hl = rawspec_gb300_fil_header_padded(h, w->pkt, kPacketBytes, (int)(off - kFrameOffset));
      }
      unsigned char *p = w->pkt + hl;
      for (int i = 0; i < nspec; i++) {
        memcpy(p, src + (size_t)i * nchans, (size_t)nchan * sizeof(float));
        p += (size_t)nchan * sizeof(float);
      }
      const size_t n = (size_t)(p - w->pkt);
      packets++;
      bytes += (long long)n;
      if (send(w->fd, w->pkt, n, 0) < 0) {
        /* ENOTCONN: no listener yet; the receiver may capture packets
         * below the socket layer, so the packet is sent once more */
        if (errno != ENOTCONN || send(w->fd, w->pkt, n, 0) < 0) errors++;
      }
      clock_gettime(CLOCK_MONOTONIC, &t1);
      const int64_t ahead = (int64_t)(8.0 * (double)bytes / w->rate) - ns_between(&t0, &t1);
      if (ahead > 100000) sleep_ns(ahead);  /* in steps of at least 100 us */
      src += nchan;
      h->fch1 += nchan * h->foff;
      chan_left -= nchan;
    }
    h->tstart += nspec * h->tsamp / 86400.0;
    spec_left -= (unsigned)nspec;
  }
  h->fch1 = fch1;
  h->nchans = nchans;
  clock_gettime(CLOCK_MONOTONIC, &t1);
  sleep_ns((int64_t)(8.0 * (double)bytes / w->rate) - ns_between(&t0, &t1));
  clock_gettime(CLOCK_MONOTONIC, &t1);
  if (errors) printf("fine channels %10d: error packets %lld/%lld\n", nchans, errors, packets);
  w->st.dumps++;
  w->st.spectra += nds;
  w->st.packets += packets;
  w->st.bytes += bytes;
  w->st.error_packets += errors;
  w->st.seconds += 1e-9 * (double)ns_between(&t0, &t1);
  return NULL;
}

RSG_EXPORT rawspec_gb300_net_writer *rawspec_gb300_net_writer_open(const rawspec_context *ctx, int product,
                                                                   const rawspec_gb300_fil_hdr *hdr, int fd,
                                                                   double rate_gbps) {
  if (!ctx || !hdr || fd < 0 || product < 0 || product >= (int)ctx->No || rate_gbps <= 0 || hdr->nchans < 1)
    return NULL;
  rawspec_gb300_net_writer *w = (rawspec_gb300_net_writer *)calloc(1, sizeof(*w));
  if (!w) return NULL;
  w->pkt = (unsigned char *)malloc(kPacketBytes);
  if (!w->pkt) {
    free(w);
    return NULL;
  }
  w->ctx = ctx;
  w->product = product;
  w->hdr = *hdr;
  w->fd = fd;
  w->rate = rate_gbps;
  return w;
}

static void join_sender(rawspec_gb300_net_writer *w) {
  if (w->thread_valid) {
    const int rc = pthread_join(w->thread, NULL);
    if (rc) fprintf(stderr, "pthread_join: %s\n", strerror(rc));
    w->thread_valid = 0;
  }
}

RSG_EXPORT int rawspec_gb300_net_writer_stats(rawspec_gb300_net_writer *w, rawspec_gb300_net_stats *st) {
  if (!w || !st) return 1;
  join_sender(w);
  *st = w->st;
  return 0;
}

RSG_EXPORT int rawspec_gb300_net_writer_close(rawspec_gb300_net_writer *w) {
  if (!w) return 0;
  join_sender(w);
  const int failed = w->st.error_packets > 0;
  free(w->pkt);
  free(w);
  return failed;
}

RSG_EXPORT void rawspec_gb300_net_dump_callback(rawspec_context *ctx, int output_product, int callback_type) {
  rawspec_gb300_net_writer **ws = (rawspec_gb300_net_writer **)ctx->user_data;
  rawspec_gb300_net_writer *w = ws ? ws[output_product] : NULL;
  if (!w) return;
  if (callback_type == RAWSPEC_CALLBACK_PRE_DUMP) {
    join_sender(w);
  } else if (callback_type == RAWSPEC_CALLBACK_POST_DUMP) {
    join_sender(w);
    const int rc = pthread_create(&w->thread, NULL, net_send, w);
    if (rc) {
      fprintf(stderr, "pthread_create: %s\n", strerror(rc));
      ctx->exit_soon = 1;
    } else {
      w->thread_valid = 1;
    }
  }
}
