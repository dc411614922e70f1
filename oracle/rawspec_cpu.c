/*
 * rawspec_cpu.c -- FP32 OpenMP CPU implementation of the reference
 * spectrometer chain (unpack -> FFT -> detect -> integrate -> FFT shift ->
 * incoherent sum), the same steps and output layout as rawspec_oracle.c but
 * in float with a precomputed-twiddle radix-2 FFT, parallel over coarse
 * channels.  The reference has no CPU path; this is the CPU baseline that
 * bench.py times on the host cores (TEST/BENCH INFRASTRUCTURE ONLY).
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "rawspec_oracle.h"

int cpu_max_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

static float snorm_f(int code, int nbits) {
  const double d = nbits == 16 ? 32767.0 : 127.0;
  double x = (double)code;
  if (x < -d) x = -d;
  return (float)(x / d);
}

/* Iterative radix-2 FFT over interleaved float complex; tw[k] = W_n^k for
 * k < n/2 (forward), brev the bit-reversal permutation. */
static void fft_f(float *z, long n, const float *tw, const long *brev, int inverse) {
  for (long i = 0; i < n; i++) {
    const long j = brev[i];
    if (i < j) {
      float tr = z[2 * i], ti = z[2 * i + 1];
      z[2 * i] = z[2 * j];
      z[2 * i + 1] = z[2 * j + 1];
      z[2 * j] = tr;
      z[2 * j + 1] = ti;
    }
  }
  const float sg = inverse ? -1.0f : 1.0f;
  for (long len = 2, step = n / 2; len <= n; len <<= 1, step >>= 1) {
    const long half = len >> 1;
    for (long i = 0; i < n; i += len) {
      float *u = z + 2 * i;
      float *v = z + 2 * (i + half);
      for (long k = 0; k < half; k++) {
        const float wr = tw[2 * k * step], wi = sg * tw[2 * k * step + 1];
        const float xr = v[2 * k] * wr - v[2 * k + 1] * wi;
        const float xi = v[2 * k] * wi + v[2 * k + 1] * wr;
        v[2 * k] = u[2 * k] - xr;
        v[2 * k + 1] = u[2 * k + 1] - xi;
        u[2 * k] += xr;
        u[2 * k + 1] += xi;
      }
    }
  }
}

static int code_at(const uint8_t *blk, int nbits, long Ntpb, int Np, int c, long t, int p, int comp) {
  const long samp = ((long)c * Ntpb + t) * Np + p;
  if (nbits == 4) {
    const uint8_t b = blk[samp];
    return comp == 0 ? (int)((int8_t)(b & 0xf0) >> 4) : (int)((int8_t)(uint8_t)(b << 4) >> 4);
  }
  if (nbits == 16) {
    const uint8_t *q = blk + 4 * samp + 2 * comp;
    return (int)(int16_t)(uint16_t)(q[0] | (q[1] << 8));
  }
  return (int)(int8_t)blk[2 * samp + comp];
}

int cpu_run(const oracle_cfg *cfg, const uint8_t *blocks, int nblocks, float **out, float **ics, int nthreads) {
  const int Nc = cfg->Nc, Np = cfg->Np, Nb = cfg->Nb;
  const long Ntpb = cfg->Ntpb;
  const long blk_bytes = oracle_block_bytes(cfg);
  const int nbuf = nblocks / Nb;
  const int Nant = cfg->Nant > 0 ? cfg->Nant : 1;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
  /* unpack tables */
  float lut8[256];
  for (int x = -128; x < 128; x++) lut8[x + 128] = snorm_f(x, 8);

  for (int i = 0; i < cfg->No; i++) {
    const long NbNtpb = (long)Nb * Ntpb;
    const long Nt = cfg->Nts[i];
    const long Nss = NbNtpb / Nt;
    long Nd = Nss / cfg->Nas[i];
    if (Nd == 0) Nd = 1;
    long Nis = cfg->Nas[i] / Nss;
    if (Nis == 0) Nis = 1;
    const int NP = abs(cfg->Npolout[i]);
    const int P = cfg->Npolout[i];
    const long dump_n = Nd * NP * Nc * Nt;
    float *acc = (float *)calloc((size_t)dump_n, sizeof(float));
    float *tw = (float *)malloc(sizeof(float) * (Nt > 1 ? Nt : 2));
    long *brev = (long *)malloc(sizeof(long) * Nt);
    for (long k = 0; k < Nt / 2; k++) {
      const double a = -2.0 * 3.14159265358979323846 * (double)k / (double)Nt;
      tw[2 * k] = (float)cos(a);
      tw[2 * k + 1] = (float)sin(a);
    }
    int lg = 0;
    while ((1L << lg) < Nt) lg++;
    for (long k = 0; k < Nt; k++) {
      long r = 0;
      for (int bit = 0; bit < lg; bit++)
        if (k & (1L << bit)) r |= 1L << (lg - 1 - bit);
      brev[k] = r;
    }
    const float sgn = cfg->conj ? -1.0f : 1.0f;
    long ndump = 0;
    for (int b = 0; b < nbuf; b++) {
#pragma omp parallel
      {
        float *x0 = (float *)malloc(sizeof(float) * 2 * Nt);
        float *x1 = (float *)malloc(sizeof(float) * 2 * Nt);
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < Nc; c++) {
          for (long s = 0; s < Nss; s++) {
            for (long n = 0; n < Nt; n++) {
              const long t = s * Nt + n;
              const uint8_t *blk = blocks + (size_t)(b * Nb + t / Ntpb) * blk_bytes;
              const long tb = t % Ntpb;
              if (cfg->nbits == 8) {
                const int8_t *q = (const int8_t *)blk + 2 * (((long)c * Ntpb + tb) * Np);
                x0[2 * n] = lut8[q[0] + 128];
                x0[2 * n + 1] = lut8[q[1] + 128];
                if (Np == 2) {
                  x1[2 * n] = lut8[q[2] + 128];
                  x1[2 * n + 1] = lut8[q[3] + 128];
                }
              } else {
                x0[2 * n] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 0), cfg->nbits);
                x0[2 * n + 1] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 1), cfg->nbits);
                if (Np == 2) {
                  x1[2 * n] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 0), cfg->nbits);
                  x1[2 * n + 1] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 1), cfg->nbits);
                }
              }
            }
            fft_f(x0, Nt, tw, brev, cfg->inverse);
            if (Np == 2) fft_f(x1, Nt, tw, brev, cfg->inverse);
            const long d = (Nis > 1) ? 0 : s / cfg->Nas[i];
            float *a0 = acc + ((d * NP + 0) * Nc + c) * Nt;
            const long pl = (long)Nc * Nt;
            for (long k = 0; k < Nt; k++) {
              const float p0 = x0[2 * k] * x0[2 * k] + x0[2 * k + 1] * x0[2 * k + 1];
              if (P == 1) {
                float p = p0;
                if (Np == 2) p += x1[2 * k] * x1[2 * k] + x1[2 * k + 1] * x1[2 * k + 1];
                a0[k] += p;
              } else {
                const float p1 = x1[2 * k] * x1[2 * k] + x1[2 * k + 1] * x1[2 * k + 1];
                const float re = x0[2 * k] * x1[2 * k] + x0[2 * k + 1] * x1[2 * k + 1];
                const float im = x0[2 * k + 1] * x1[2 * k] - x0[2 * k] * x1[2 * k + 1];
                if (P == 4) {
                  a0[k] += p0;
                  a0[pl + k] += p1;
                } else {
                  a0[k] += p0 + p1;
                  a0[pl + k] += p0 - p1;
                }
                a0[2 * pl + k] += re;
                a0[3 * pl + k] += sgn * im;
              }
            }
          }
        }
        free(x0);
        free(x1);
      }
      if ((b + 1) % Nis == 0) {
        float *dst = out[i] + ndump * dump_n;
        for (long r = 0; r < Nd * NP * Nc; r++)
          for (long k = 0; k < Nt; k++) dst[r * Nt + (k + Nt / 2) % Nt] = acc[r * Nt + k];
        if (cfg->ics && ics && ics[i]) {
          const int Nca = Nc / Nant;
          float *idst = ics[i] + ndump * (dump_n / Nant);
          for (long dp = 0; dp < Nd * NP; dp++)
            for (int cc = 0; cc < Nca; cc++)
              for (long k = 0; k < Nt; k++) {
                float sum = 0;
                for (int a = 0; a < Nant; a++) sum = fmaf(cfg->weights[a], dst[(dp * Nc + a * Nca + cc) * Nt + k], sum);
                idst[(dp * Nca + cc) * Nt + k] = sum;
              }
        }
        memset(acc, 0, sizeof(float) * dump_n);
        ndump++;
      }
    }
    free(acc);
    free(tw);
    free(brev);
  }
  return 0;
}
