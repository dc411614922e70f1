/*
 * rawspec_cpu.c -- FP32 OpenMP CPU implementation of the reference
 * spectrometer chain (unpack -> FFT -> detect -> integrate -> FFT shift ->
 * incoherent sum), the same steps and output layout as rawspec_oracle.c but
 * in float with a Stockham radix-4 FFT (four-step above 16384 points, so
 * that every sub-transform works in cache), parallel over coarse channels.  The reference has no CPU path; this is the CPU baseline that
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

/* ---- FFT: Stockham radix-4 (radix-2 for an odd power of two), and a
 * four-step split for long transforms, over interleaved float complex ---- */

typedef struct {
  long n;
  int nst;          /* stages */
  int radix[32];
  long ns[32];      /* length of the sub-transforms already done before the stage */
  float *tw[32];    /* stage twiddles [(r-1)*ns + k] = W_(ns*R)^(r k), forward, k < ns */
} stock_plan;

static void stock_plan_init(stock_plan *p, long n) {
  p->n = n;
  p->nst = 0;
  long ns = 1;
  while (ns < n) {
    const int R = (n / ns) % 4 == 0 ? 4 : 2;
    p->radix[p->nst] = R;
    p->ns[p->nst] = ns;
    float *t = (float *)malloc(sizeof(float) * 2 * (size_t)(R - 1) * (size_t)ns);
    for (int r = 1; r < R; r++)
      for (long k = 0; k < ns; k++) {
        const double a = -2.0 * 3.14159265358979323846 * (double)(r * k) / (double)(ns * R);
        t[2 * ((r - 1) * ns + k)] = (float)cos(a);
        t[2 * ((r - 1) * ns + k) + 1] = (float)sin(a);
      }
    p->tw[p->nst++] = t;
    ns *= R;
  }
}

static void stock_plan_free(stock_plan *p) {
  for (int i = 0; i < p->nst; i++) free(p->tw[i]);
}

/* One transform of x (length p->n) with y as work space; returns the buffer
 * that holds the result (x or y).  sg = +1 forward, -1 inverse. */
static float *stock_fft(const stock_plan *p, float *restrict x, float *restrict y, float sg) {
  const long n = p->n;
  for (int st = 0; st < p->nst; st++) {
    const int R = p->radix[st];
    const long ns = p->ns[st], T = n / R;
    const float *restrict tw = p->tw[st];
    for (long hi = 0; hi < T / ns; hi++) {
      const float *restrict xs = x + 2 * hi * ns;
      float *restrict ys = y + 2 * hi * ns * R;
      if (R == 4) {
        for (long k = 0; k < ns; k++) {
          float ar = xs[2 * k], ai = xs[2 * k + 1];
          float br = xs[2 * (k + T)], bi = xs[2 * (k + T) + 1];
          float cr = xs[2 * (k + 2 * T)], ci = xs[2 * (k + 2 * T) + 1];
          float dr = xs[2 * (k + 3 * T)], di = xs[2 * (k + 3 * T) + 1];
          {
            float wr = tw[2 * k], wi = sg * tw[2 * k + 1], t;
            t = br * wr - bi * wi; bi = br * wi + bi * wr; br = t;
            wr = tw[2 * (ns + k)]; wi = sg * tw[2 * (ns + k) + 1];
            t = cr * wr - ci * wi; ci = cr * wi + ci * wr; cr = t;
            wr = tw[2 * (2 * ns + k)]; wi = sg * tw[2 * (2 * ns + k) + 1];
            t = dr * wr - di * wi; di = dr * wi + di * wr; dr = t;
          }
          const float t0r = ar + cr, t0i = ai + ci, t1r = ar - cr, t1i = ai - ci;
          const float t2r = br + dr, t2i = bi + di, t3r = br - dr, t3i = bi - di;
          /* X1 = t1 - sg i t3, X3 = t1 + sg i t3 */
          ys[2 * k] = t0r + t2r;
          ys[2 * k + 1] = t0i + t2i;
          ys[2 * (k + ns)] = t1r + sg * t3i;
          ys[2 * (k + ns) + 1] = t1i - sg * t3r;
          ys[2 * (k + 2 * ns)] = t0r - t2r;
          ys[2 * (k + 2 * ns) + 1] = t0i - t2i;
          ys[2 * (k + 3 * ns)] = t1r - sg * t3i;
          ys[2 * (k + 3 * ns) + 1] = t1i + sg * t3r;
        }
      } else {
        for (long k = 0; k < ns; k++) {
          const float ar = xs[2 * k], ai = xs[2 * k + 1];
          float br = xs[2 * (k + T)], bi = xs[2 * (k + T) + 1];
          if (ns > 1) {
            const float wr = tw[2 * k], wi = sg * tw[2 * k + 1], t = br * wr - bi * wi;
            bi = br * wi + bi * wr;
            br = t;
          }
          ys[2 * k] = ar + br;
          ys[2 * k + 1] = ai + bi;
          ys[2 * (k + ns)] = ar - br;
          ys[2 * (k + ns) + 1] = ai - bi;
        }
      }
    }
    float *t = x;
    x = y;
    y = t;
  }
  return x;
}

/* Transforms above kFourStep points take the four-step split N = N1 * N2
 * (x[n1 + N1 n2] -> X[k2 + N2 k1]): N2-point transforms of blocks of kColBlk
 * gathered columns, twiddled by W_N^(n1 k2) into Y[k2][n1], N1-point
 * transforms of the rows of Y, and a blocked transpose into X. */
enum { kFourStep = 16384, kColBlk = 8, kTrBlk = 16 };

typedef struct {
  long n, n1, n2;
  stock_plan direct, p1, p2;
  float *tw;        /* W_N^(n1 k2) [k2][n1], forward */
} cpu_fft;

static void cpu_fft_init(cpu_fft *f, long n) {
  f->n = n;
  f->tw = NULL;
  if (n <= kFourStep) {
    stock_plan_init(&f->direct, n);
    return;
  }
  int lg = 0;
  while ((1L << lg) < n) lg++;
  f->n1 = 1L << (lg / 2);
  f->n2 = n / f->n1;
  stock_plan_init(&f->p1, f->n1);
  stock_plan_init(&f->p2, f->n2);
  f->tw = (float *)malloc(sizeof(float) * 2 * (size_t)n);
  for (long k2 = 0; k2 < f->n2; k2++)
    for (long a = 0; a < f->n1; a++) {
      const double ang = -2.0 * 3.14159265358979323846 * (double)((a * k2) % n) / (double)n;
      f->tw[2 * (k2 * f->n1 + a)] = (float)cos(ang);
      f->tw[2 * (k2 * f->n1 + a) + 1] = (float)sin(ang);
    }
}

static void cpu_fft_free(cpu_fft *f) {
  if (f->n <= kFourStep) {
    stock_plan_free(&f->direct);
    return;
  }
  stock_plan_free(&f->p1);
  stock_plan_free(&f->p2);
  free(f->tw);
}

/* Floats of work space a transform needs besides its data. */
static long cpu_fft_work(const cpu_fft *f) {
  if (f->n <= kFourStep) return 2 * f->n;
  return 2 * f->n + 2 * (kColBlk + 1) * f->n2 + 2 * f->n1;
}

/* Transforms x (length n) in place; work holds cpu_fft_work(f) floats. */
static void cpu_fft_run(const cpu_fft *f, float *x, float *work, int inverse) {
  const float sg = inverse ? -1.0f : 1.0f;
  const long n = f->n;
  if (n <= kFourStep) {
    float *r = stock_fft(&f->direct, x, work, sg);
    if (r != x) memcpy(x, r, sizeof(float) * 2 * (size_t)n);
    return;
  }
  const long n1 = f->n1, n2 = f->n2;
  float *Y = work;                       /* [k2][n1] */
  float *cb = work + 2 * n;              /* kColBlk gathered columns, then a spare one */
  float *rw = cb + 2 * (kColBlk + 1) * n2;  /* row work space */
  for (long c0 = 0; c0 < n1; c0 += kColBlk) {
    const int nb = (int)(n1 - c0 < kColBlk ? n1 - c0 : kColBlk);
    for (long b2 = 0; b2 < n2; b2++)
      for (int b = 0; b < nb; b++) {
        cb[2 * (b * n2 + b2)] = x[2 * (c0 + b + n1 * b2)];
        cb[2 * (b * n2 + b2) + 1] = x[2 * (c0 + b + n1 * b2) + 1];
      }
    for (int b = 0; b < nb; b++) {
      float *col = cb + 2 * b * n2;
      float *r = stock_fft(&f->p2, col, cb + 2 * kColBlk * n2, sg);
      if (r != col) memcpy(col, r, sizeof(float) * 2 * (size_t)n2);
    }
    for (long k2 = 0; k2 < n2; k2++)
      for (int b = 0; b < nb; b++) {
        const float vr = cb[2 * (b * n2 + k2)], vi = cb[2 * (b * n2 + k2) + 1];
        const float wr = f->tw[2 * (k2 * n1 + c0 + b)], wi = sg * f->tw[2 * (k2 * n1 + c0 + b) + 1];
        Y[2 * (k2 * n1 + c0 + b)] = vr * wr - vi * wi;
        Y[2 * (k2 * n1 + c0 + b) + 1] = vr * wi + vi * wr;
      }
  }
  for (long k2 = 0; k2 < n2; k2++) {
    float *row = Y + 2 * k2 * n1;
    float *r = stock_fft(&f->p1, row, rw, sg);
    if (r != row) memcpy(row, r, sizeof(float) * 2 * (size_t)n1);
  }
  /* X[k2 + N2 k1] = Y[k2][k1] */
  for (long k2b = 0; k2b < n2; k2b += kTrBlk)
    for (long k1b = 0; k1b < n1; k1b += kTrBlk)
      for (long k2 = k2b; k2 < k2b + kTrBlk && k2 < n2; k2++)
        for (long k1 = k1b; k1 < k1b + kTrBlk && k1 < n1; k1++) {
          x[2 * (k2 + n2 * k1)] = Y[2 * (k2 * n1 + k1)];
          x[2 * (k2 + n2 * k1) + 1] = Y[2 * (k2 * n1 + k1) + 1];
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
    cpu_fft plan;
    cpu_fft_init(&plan, Nt);
    const float sgn = cfg->conj ? -1.0f : 1.0f;
    long ndump = 0;
    for (int b = 0; b < nbuf; b++) {
#pragma omp parallel
      {
        float *x0 = (float *)malloc(sizeof(float) * 2 * Nt);
        float *x1 = (float *)malloc(sizeof(float) * 2 * Nt);
        float *work = (float *)malloc(sizeof(float) * (size_t)cpu_fft_work(&plan));
#pragma omp for schedule(dynamic, 1)
        for (int c = 0; c < Nc; c++) {
          for (long s = 0; s < Nss; s++) {
            /* the spectrum's samples, one run per block it spans */
            for (long n = 0; n < Nt;) {
              const long t = s * Nt + n;
              const uint8_t *blk = blocks + (size_t)(b * Nb + t / Ntpb) * blk_bytes;
              const long tb0 = t % Ntpb;
              const long run = Nt - n < Ntpb - tb0 ? Nt - n : Ntpb - tb0;
              if (cfg->nbits == 8) {
                const int8_t *q = (const int8_t *)blk + 2 * (((long)c * Ntpb + tb0) * Np);
                for (long m = 0; m < run; m++, q += 2 * Np) {
                  x0[2 * (n + m)] = lut8[q[0] + 128];
                  x0[2 * (n + m) + 1] = lut8[q[1] + 128];
                  if (Np == 2) {
                    x1[2 * (n + m)] = lut8[q[2] + 128];
                    x1[2 * (n + m) + 1] = lut8[q[3] + 128];
                  }
                }
              } else {
                for (long m = 0; m < run; m++) {
                  const long tb = tb0 + m;
                  x0[2 * (n + m)] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 0), cfg->nbits);
                  x0[2 * (n + m) + 1] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 0, 1), cfg->nbits);
                  if (Np == 2) {
                    x1[2 * (n + m)] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 0), cfg->nbits);
                    x1[2 * (n + m) + 1] = snorm_f(code_at(blk, cfg->nbits, Ntpb, Np, c, tb, 1, 1), cfg->nbits);
                  }
                }
              }
              n += run;
            }
            cpu_fft_run(&plan, x0, work, cfg->inverse);
            if (Np == 2) cpu_fft_run(&plan, x1, work, cfg->inverse);
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
        free(work);
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
    cpu_fft_free(&plan);
  }
  return 0;
}
