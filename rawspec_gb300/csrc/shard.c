/*
 * shard.c -- channel shards of one observation for several GPUs.
 *
 * The spectrometer's outputs of a coarse channel depend on that channel's
 * voltages only, and the weighted incoherent sum on the antennas of one
 * channel-within-antenna.  A shard is therefore a contiguous range
 * [k0, k0 + nk) of channels-within-antenna taken from every antenna; it is
 * processed by an ordinary context of Nant * nk channels (one per GPU, one
 * process per GPU) with no data exchanged between shards.  The reference
 * runs one process per GPU on whole observations (rawspec.c:292-295); these
 * helpers split one observation's channels instead and put the shards'
 * dumps back in the full layout.
 *
 * Host code only: nothing here touches a GPU.
 */
#include <stddef.h>
#include <string.h>

#include "rawspec.h"
#include "rawspec_gb300.h"

#define RSG_EXPORT __attribute__((visibility("default")))

RSG_EXPORT int rawspec_gb300_shard_range(unsigned int Nc, unsigned int Nant, int rank, int world,
                                         unsigned int *k0, unsigned int *nk) {
  if (Nant == 0) Nant = 1;
  if (!k0 || !nk || Nc == 0 || Nc % Nant != 0 || world < 1 || rank < 0 || rank >= world) return 1;
  const unsigned long long nca = Nc / Nant;
  const unsigned long long lo = nca * (unsigned long long)rank / (unsigned long long)world;
  const unsigned long long hi = nca * (unsigned long long)(rank + 1) / (unsigned long long)world;
  if (hi <= lo) return 1;
  *k0 = (unsigned int)lo;
  *nk = (unsigned int)(hi - lo);
  return 0;
}

RSG_EXPORT int rawspec_gb300_shard_context(const rawspec_context *full, int rank, int world, rawspec_context *shard) {
  unsigned int k0 = 0, nk = 0;
  if (!full || !shard) return 1;
  const unsigned int nant = full->Nant == 0 ? 1 : full->Nant;
  if (rawspec_gb300_shard_range(full->Nc, nant, rank, world, &k0, &nk) != 0) return 1;
  memset(shard, 0, sizeof(*shard));
  shard->No = full->No;
  shard->Np = full->Np;
  shard->Nant = full->Nant;
  shard->Nc = nant * nk;
  shard->Ntpb = full->Ntpb;
  shard->Nbc = 0;
  shard->Nbps = full->Nbps;
  for (int i = 0; i < MAX_OUTPUTS; i++) {
    shard->Npolout[i] = full->Npolout[i];
    shard->Nts[i] = full->Nts[i];
    shard->Nas[i] = full->Nas[i];
  }
  shard->dump_callback = full->dump_callback;
  shard->user_data = full->user_data;
  shard->Nb = full->Nb;
  shard->gpu_index = full->gpu_index;
  shard->input_conjugated = full->input_conjugated;
  shard->incoherently_sum = full->incoherently_sum;
  shard->Naws = full->Naws;
  shard->Aws = full->Aws;
  return 0;
}

RSG_EXPORT int rawspec_gb300_shard_fill_block(const void *full_block, unsigned int Nc, unsigned int Nant,
                                              unsigned int k0, unsigned int nk, size_t channel_bytes,
                                              void *shard_block) {
  if (Nant == 0) Nant = 1;
  if (!full_block || !shard_block || Nc % Nant != 0 || nk == 0 || k0 + nk > Nc / Nant) return 1;
  const unsigned int nca = Nc / Nant;
  const char *src = (const char *)full_block;
  char *dst = (char *)shard_block;
  for (unsigned int a = 0; a < Nant; a++)
    memcpy(dst + (size_t)a * nk * channel_bytes, src + ((size_t)a * nca + k0) * channel_bytes,
           (size_t)nk * channel_bytes);
  return 0;
}

RSG_EXPORT int rawspec_gb300_shard_place_dump(const float *shard_dump, unsigned int Nc, unsigned int Nant,
                                              unsigned int k0, unsigned int nk, unsigned int rows, unsigned int Nt,
                                              int ics, float *full_dump) {
  if (Nant == 0) Nant = 1;
  if (!shard_dump || !full_dump || Nc % Nant != 0 || nk == 0 || k0 + nk > Nc / Nant || Nt == 0) return 1;
  const unsigned int nca = Nc / Nant;
  /* rows: Nd * |Npolout|; a row holds the channels of one spectrum and plane */
  const unsigned int groups = ics ? 1 : Nant;          /* antenna runs per row */
  const unsigned int shard_row = groups * nk, full_row = ics ? nca : Nc;
  for (unsigned int r = 0; r < rows; r++)
    for (unsigned int a = 0; a < groups; a++)
      memcpy(full_dump + ((size_t)r * full_row + (size_t)a * nca + k0) * Nt,
             shard_dump + ((size_t)r * shard_row + (size_t)a * nk) * Nt, (size_t)nk * Nt * sizeof(float));
  return 0;
}
