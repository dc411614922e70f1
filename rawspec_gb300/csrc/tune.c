/* tune.c -- the tuning table: kernel choices per (FFT length, sample bits,
 * Npolout), written by the tuner (rawspec_gb300.tune, which times whole
 * buffers of the caller's configuration with each candidate) and read by
 * rawspec_initialize and the device-memory estimate from the file named by
 * RAWSPEC_GB300_TUNE_FILE.
 *
 * One entry per line, '#' starts a comment:
 *     <nfft> <nbits> <npolout> [dft=tc|cuda] [ctas=N] [lag=N] [ring=N]
 * nbits is the width of the samples the kernels read (4-bit input is
 * expanded to 8 bits first).  A later line for the same triple replaces
 * the earlier one.  Malformed lines are reported on stderr and skipped. */
#include <errno.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "rawspec_gb300.h"

#define RSG_EXPORT __attribute__((visibility("default")))

static void tune_unset(rawspec_gb300_tune *t) {
  t->dft = -1;
  t->ctas = 0;
  t->lag = 0;
  t->ring = 0;
}

static int parse_int(const char *s, int lo, int hi, int *v) {
  char *end = NULL;
  errno = 0;
  const long x = strtol(s, &end, 10);
  if (errno || end == s || *end != '\0' || x < lo || x > hi) return 1;
  *v = (int)x;
  return 0;
}

/* Parses one line; 1 and the entry if it holds one, 0 for a blank or
 * comment line, -1 if malformed. */
static int parse_line(char *line, unsigned *nfft, int *nbits, int *npolout, rawspec_gb300_tune *t) {
  char *hash = strchr(line, '#');
  if (hash) *hash = '\0';
  char *save = NULL;
  char *tok = strtok_r(line, " \t\r\n", &save);
  if (!tok) return 0;
  int n = 0;
  if (parse_int(tok, 1, 1 << 24, &n)) return -1;
  *nfft = (unsigned)n;
  tok = strtok_r(NULL, " \t\r\n", &save);
  if (!tok || parse_int(tok, 4, 16, nbits)) return -1;
  tok = strtok_r(NULL, " \t\r\n", &save);
  if (!tok || parse_int(tok, -4, 4, npolout)) return -1;
  tune_unset(t);
  while ((tok = strtok_r(NULL, " \t\r\n", &save)) != NULL) {
    char *eq = strchr(tok, '=');
    if (!eq) return -1;
    *eq = '\0';
    const char *val = eq + 1;
    if (strcmp(tok, "dft") == 0) {
      if (strcmp(val, "tc") == 0) t->dft = 1;
      else if (strcmp(val, "cuda") == 0) t->dft = 0;
      else return -1;
    } else if (strcmp(tok, "ctas") == 0) {
      if (parse_int(val, 1, 64, &t->ctas)) return -1;
    } else if (strcmp(tok, "lag") == 0) {
      if (parse_int(val, 1, 64, &t->lag)) return -1;
    } else if (strcmp(tok, "ring") == 0) {
      if (parse_int(val, 2, 128, &t->ring)) return -1;
    } else {
      return -1;
    }
  }
  if (t->lag > 0 && t->ring > 0 && t->ring <= t->lag) return -1;
  return 1;
}

RSG_EXPORT int rawspec_gb300_tune_lookup(unsigned nfft, int nbits, int npolout, rawspec_gb300_tune *t) {
  if (!t) return -1;
  tune_unset(t);
  const char *path = getenv("RAWSPEC_GB300_TUNE_FILE");
  if (!path || !path[0]) return 0;
  FILE *f = fopen(path, "r");
  if (!f) {
    fprintf(stderr, "tuning table %s: %s\n", path, strerror(errno));
    return -1;
  }
  char line[512];
  int found = 0, lineno = 0;
  while (fgets(line, sizeof(line), f)) {
    lineno++;
    unsigned n = 0;
    int b = 0, p = 0;
    rawspec_gb300_tune e;
    const int r = parse_line(line, &n, &b, &p, &e);
    if (r < 0) {
      fprintf(stderr, "tuning table %s:%d: malformed entry skipped\n", path, lineno);
      continue;
    }
    if (r > 0 && n == nfft && b == nbits && p == npolout) {
      *t = e;
      found = 1;
    }
  }
  fclose(f);
  return found;
}
