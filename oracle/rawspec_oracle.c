/*
 * rawspec_oracle.c -- FP64 CPU restatement of the reference spectrometer
 * chain.  TEST INFRASTRUCTURE ONLY: used by tests/, __graft_entry__.smoke()
 * and bench.py's CPU-baseline leg as the checker; never linked into or
 * called by the library.
 *
 * It follows the reference's device path step by step:
 *   - block corner turn: spectrum s of channel c covers time samples
 *     [s*Nt, (s+1)*Nt) of the channel's Nb*Ntpb concatenated samples
 *     (rawspec_gpu.cu:1182-1195 plan strides, :1454-1460 copy);
 *   - unpack: texture SNORM read, x / 127 (8 bit) or x / 32767 (16 bit),
 *     the most negative code clamped to -1 (rawspec_gpu.cu:133-148, :845-866),
 *     rounded to float as the FP32 FFT sees it;  4-bit input is first expanded
 *     to int8 with the high nibble as the real part (rawspec_gpu.cu:342-374);
 *   - FFT: forward exp(-2 pi i k n / N) for fft_dir > 0, inverse otherwise,
 *     unnormalised (rawspec_gpu.cu:1560-1563), computed here in double;
 *   - detection (rawspec_gpu.cu:153-267): total power, full pol
 *     (XX, YY, Re XY*, Im XY*) or Stokes (I, Q, U, V), Im/V negated for
 *     conjugated input;
 *   - integration over Nas[i] consecutive spectra, across input buffers when
 *     Nts*Nas exceeds the buffer (rawspec_gpu.cu:297-318, :1572);
 *   - FFT shift and dump layout [Nd][|P|][Nc][Nt] (rawspec_gpu.cu:1647-1697);
 *   - weighted incoherent sum over antennas, [Nd][|P|][Nc/Nant][Nt]
 *     (rawspec_gpu.cu:321-340, :1603-1633).
 *
 * Parity pins: the known-answer tests of tests/test_oracle.py (the impulse
 * case of the reference's own rawspectest.c, single tones, Stokes identities)
 * and exhaustive checks of the unpack against exact rational rounding.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "rawspec_oracle.h"

static const double kPi = 3.14159265358979323846264338327950288;

/* Unpack of one component code, as the FP32 FFT input of the reference. */
double oracle_snorm(int code, int nbits) {
  const double d = nbits == 16 ? 32767.0 : 127.0;
  double x = (double)code;
  if (x < -d) x = -d;
  return (double)(float)(x / d);
}

/* In-place FFT of n complex doubles (re/im interleaved).  Powers of two use
 * an iterative radix-2 decimation in time; other lengths a direct DFT. */
void oracle_fft(double *z, long n, int inverse) {
  const double sgn = inverse ? 1.0 : -1.0;
  if (n <= 1) return;
  if ((n & (n - 1)) != 0) {
    double *t = (double *)malloc(sizeof(double) * 2 * n);
    for (long k = 0; k < n; k++) {
      double sr = 0, si = 0;
      for (long m = 0; m < n; m++) {
        const double a = sgn * 2.0 * kPi * (double)((k * m) % n) / (double)n;
        const double c = cos(a), s = sin(a);
        sr += z[2 * m] * c - z[2 * m + 1] * s;
        si += z[2 * m] * s + z[2 * m + 1] * c;
      }
      t[2 * k] = sr;
      t[2 * k + 1] = si;
    }
    memcpy(z, t, sizeof(double) * 2 * n);
    free(t);
    return;
  }
  /* bit reversal */
  for (long i = 1, j = 0; i < n; i++) {
    long bit = n >> 1;
    for (; j & bit; bit >>= 1) j ^= bit;
    j ^= bit;
    if (i < j) {
      double tr = z[2 * i], ti = z[2 * i + 1];
      z[2 * i] = z[2 * j];
      z[2 * i + 1] = z[2 * j + 1];
      z[2 * j] = tr;
      z[2 * j + 1] = ti;
    }
  }
  for (long len = 2; len <= n; len <<= 1) {
    const long half = len >> 1;
    for (long k = 0; k < half; k++) {
      const double a = sgn * 2.0 * kPi * (double)k / (double)len;
      const double wr = cos(a), wi = sin(a);
      for (long i = 0; i < n; i += len) {
        double *u = z + 2 * (i + k), *v = z + 2 * (i + k + half);
        const double xr = v[0] * wr - v[1] * wi;
        const double xi = v[0] * wi + v[1] * wr;
        v[0] = u[0] - xr;
        v[1] = u[1] - xi;
        u[0] += xr;
        u[1] += xi;
      }
    }
  }
}

/* Code of component `comp` (0 re, 1 im) of pol p, time t, channel c, in a
 * host block laid out [chan][time][pol][re,im]. */
static int block_code(const uint8_t *blk, int nbits, long Ntpb, int Np, int c, long t, int p, int comp) {
  const long samp = ((long)c * Ntpb + t) * Np + p; /* complex sample index */
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

long oracle_block_bytes(const oracle_cfg *cfg) {
  const long samples = (long)cfg->Nc * cfg->Ntpb * cfg->Np;
  return cfg->nbits == 4 ? samples : samples * 2 * (cfg->nbits / 8);
}

static void derived(const oracle_cfg *cfg, int i, long *Nss, long *Nis, long *Nd) {
  const long NbNtpb = (long)cfg->Nb * cfg->Ntpb;
  *Nss = NbNtpb / cfg->Nts[i];
  *Nd = *Nss / cfg->Nas[i];
  if (*Nd == 0) *Nd = 1;
  *Nis = cfg->Nas[i] / *Nss;
  if (*Nis == 0) *Nis = 1;
}

long oracle_dump_doubles(const oracle_cfg *cfg, int i) {
  long Nss, Nis, Nd;
  derived(cfg, i, &Nss, &Nis, &Nd);
  return Nd * (long)abs(cfg->Npolout[i]) * cfg->Nc * cfg->Nts[i];
}

long oracle_num_dumps(const oracle_cfg *cfg, int i, int nbuf) {
  long Nss, Nis, Nd;
  derived(cfg, i, &Nss, &Nis, &Nd);
  return nbuf / Nis;
}

/* Accumulates the detected bins of one spectrum (both pols) into acc
 * ([|P|][Nt] for this channel/integration). */
static void detect(const oracle_cfg *cfg, int i, const double *x0, const double *x1, double *acc, long Nt) {
  const int P = cfg->Npolout[i];
  const double sgn = cfg->conj ? -1.0 : 1.0;
  for (long k = 0; k < Nt; k++) {
    const double p0 = x0[2 * k] * x0[2 * k] + x0[2 * k + 1] * x0[2 * k + 1];
    if (P == 1) {
      double p = p0;
      if (cfg->Np == 2) p += x1[2 * k] * x1[2 * k] + x1[2 * k + 1] * x1[2 * k + 1];
      acc[k] += p;
      continue;
    }
    const double p1 = x1[2 * k] * x1[2 * k] + x1[2 * k + 1] * x1[2 * k + 1];
    const double re = x0[2 * k] * x1[2 * k] + x0[2 * k + 1] * x1[2 * k + 1];
    const double im = x0[2 * k + 1] * x1[2 * k] - x0[2 * k] * x1[2 * k + 1];
    if (P == 4) {
      acc[k] += p0;
      acc[Nt + k] += p1;
    } else {
      acc[k] += p0 + p1;
      acc[Nt + k] += p0 - p1;
    }
    acc[2 * Nt + k] += re;
    acc[3 * Nt + k] += sgn * im;
  }
}

int oracle_run(const oracle_cfg *cfg, const uint8_t *blocks, int nblocks, double **out, double **ics) {
  const int Nc = cfg->Nc, Np = cfg->Np, Nb = cfg->Nb;
  const long Ntpb = cfg->Ntpb;
  const long blk_bytes = oracle_block_bytes(cfg);
  const int nbuf = nblocks / Nb;
  const long Tbuf = (long)Nb * Ntpb;
  const int Nant = cfg->Nant > 0 ? cfg->Nant : 1;

  for (int i = 0; i < cfg->No; i++) {
    long Nss, Nis, Nd;
    derived(cfg, i, &Nss, &Nis, &Nd);
    const long Nt = cfg->Nts[i];
    const int NP = abs(cfg->Npolout[i]);
    const long dump_n = Nd * NP * Nc * Nt;
    /* integration state [Nd][NP][Nc][Nt], unshifted */
    double *acc = (double *)calloc((size_t)dump_n, sizeof(double));
    double *x0 = (double *)malloc(sizeof(double) * 2 * Nt);
    double *x1 = (double *)malloc(sizeof(double) * 2 * Nt);
    double *tmp = (double *)malloc(sizeof(double) * NP * Nt);
    long ndump = 0;
    for (int b = 0; b < nbuf; b++) {
      for (int c = 0; c < Nc; c++) {
        for (long s = 0; s < Nss; s++) {
          for (long n = 0; n < Nt; n++) {
            const long t = s * Nt + n; /* time within the buffer */
            const uint8_t *blk = blocks + (size_t)(b * Nb + t / Ntpb) * blk_bytes;
            const long tb = t % Ntpb;
            x0[2 * n] = oracle_snorm(block_code(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 0), cfg->nbits);
            x0[2 * n + 1] = oracle_snorm(block_code(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 1), cfg->nbits);
            if (Np == 2) {
              x1[2 * n] = oracle_snorm(block_code(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 0), cfg->nbits);
              x1[2 * n + 1] = oracle_snorm(block_code(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 1), cfg->nbits);
            }
          }
          oracle_fft(x0, Nt, cfg->inverse);
          if (Np == 2) oracle_fft(x1, Nt, cfg->inverse);
          const long d = (Nis > 1) ? 0 : s / cfg->Nas[i];
          memset(tmp, 0, sizeof(double) * NP * Nt);
          detect(cfg, i, x0, x1, tmp, Nt);
          for (int p = 0; p < NP; p++)
            for (long k = 0; k < Nt; k++) acc[((d * NP + p) * Nc + c) * Nt + k] += tmp[p * Nt + k];
        }
      }
      if ((b + 1) % Nis == 0) {
        /* dump: FFT shift */
        double *dst = out[i] + ndump * dump_n;
        for (long r = 0; r < Nd * NP * Nc; r++)
          for (long k = 0; k < Nt; k++) dst[r * Nt + (k + Nt / 2) % Nt] = acc[r * Nt + k];
        if (cfg->ics && ics && ics[i]) {
          const int Nca = Nc / Nant;
          double *idst = ics[i] + ndump * (dump_n / Nant);
          for (long dp = 0; dp < Nd * NP; dp++)
            for (int cc = 0; cc < Nca; cc++)
              for (long k = 0; k < Nt; k++) {
                double sum = 0;
                for (int a = 0; a < Nant; a++) sum += (double)cfg->weights[a] * dst[(dp * Nc + a * Nca + cc) * Nt + k];
                idst[(dp * Nca + cc) * Nt + k] = sum;
              }
        }
        memset(acc, 0, sizeof(double) * dump_n);
        ndump++;
      }
    }
    free(acc);
    free(x0);
    free(x1);
    free(tmp);
  }
  return 0;
}
