/*
 * rawspec_oracle.h -- CPU restatements of the reference spectrometer chain.
 * TEST INFRASTRUCTURE ONLY (tests/, __graft_entry__.smoke(), bench.py's CPU
 * baseline leg).  See rawspec_oracle.c (FP64 checker) and rawspec_cpu.c
 * (FP32 OpenMP chain timed as the CPU baseline).
 */
#ifndef RAWSPEC_ORACLE_H
#define RAWSPEC_ORACLE_H

#include <stdint.h>

typedef struct {
  int Nc, Np, Ntpb, Nb; /* channels, pols, samples per block, blocks per buffer */
  int nbits;            /* 4, 8 or 16 (host block format) */
  int Nant;             /* antennas (channels grouped per antenna) */
  int No;               /* products */
  int Nts[4], Nas[4], Npolout[4];
  int conj;             /* input conjugated: negate Im XY* / V */
  int inverse;          /* 1: inverse FFT (fft_dir <= 0) */
  int ics;              /* 1: weighted incoherent sum */
  const float *weights; /* Nant weights */
} oracle_cfg;

/* Bytes of one host block. */
long oracle_block_bytes(const oracle_cfg *cfg);
/* Values per dump of product i ([Nd][|P|][Nc][Nt]). */
long oracle_dump_doubles(const oracle_cfg *cfg, int i);
/* Dumps produced by nbuf buffers for product i. */
long oracle_num_dumps(const oracle_cfg *cfg, int i, int nbuf);
/* FP32-as-seen unpack of one code. */
double oracle_snorm(int code, int nbits);
/* In-place double FFT. */
void oracle_fft(double *z, long n, int inverse);

/* FP64 run over nblocks host blocks; out[i] receives num_dumps*dump_doubles
 * values, ics[i] (if cfg->ics) num_dumps*dump_doubles/Nant. */
int oracle_run(const oracle_cfg *cfg, const uint8_t *blocks, int nblocks, double **out, double **ics);

/* FP32 OpenMP run of the same chain (same outputs, in float), nthreads
 * threads (0 = all). */
int cpu_run(const oracle_cfg *cfg, const uint8_t *blocks, int nblocks, float **out, float **ics, int nthreads);
/* Threads cpu_run would use for nthreads = 0. */
int cpu_max_threads(void);

#endif
