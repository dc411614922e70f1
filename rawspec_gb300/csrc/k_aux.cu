// k_aux.cu -- plan-time twiddle tables, 4-bit expansion, the weighted
// incoherent sum across antennas and the compensated integration step.
#include <algorithm>
#include <cstdint>

#include "common.cuh"
#include "internal.h"

namespace rsg {

// W_n^(m*stride) = exp(-2 pi i m stride / n), FP64 sincospi rounded to float.
// Used only when a context is initialised.
__global__ void k_twiddle(float2* dst, long long count, long long n, long long stride) {
  for (long long m = blockIdx.x * (long long)blockDim.x + threadIdx.x; m < count;
       m += (long long)gridDim.x * blockDim.x) {
    const long long e = (m * stride) % n;
    double s, c;
    sincospi(2.0 * (double)e / (double)n, &s, &c);
    dst[m] = make_float2((float)c, (float)(-s));
  }
}

cudaError_t twiddle_fill(float2* dst, long long count, long long n, long long stride, cudaStream_t s) {
  const int blocks = (int)std::min<long long>((count + 255) / 256, 4096);
  k_twiddle<<<std::max(blocks, 1), 256, 0, s>>>(dst, count, n, stride);
  return cudaGetLastError();
}

__device__ __forceinline__ float2 w_of(long long e, long long n) {
  double s, c;
  sincospi(2.0 * (double)e / (double)n, &s, &c);
  return make_float2((float)c, (float)(-s));
}

// Pass-ordered twiddle table of a GroupFFT<N, R> (layout in fft_core.cuh):
// full passes p >= 1 with Ns = R^p hold [r-1][k] = W_N^(k r N/(Ns R)); the
// trailing pass of radix RL holds [r-1][b] = W_N^(b r).
__global__ void k_stockham_twiddle(float2* dst, int N, int R, int size) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= size) return;
  int off = 0, Ns = R;
  while (Ns * R <= N) {  // full passes 1 .. FULL-1
    const int blk = (R - 1) * Ns;
    if (i < off + blk) {
      const int r = (i - off) / Ns + 1, k = (i - off) % Ns;
      dst[i] = w_of((long long)k * r * (N / (Ns * R)), N);
      return;
    }
    off += blk;
    Ns *= R;
  }
  const int rl = N / Ns;  // trailing pass
  const int nsl = N / rl;
  const int r = (i - off) / nsl + 1, b = (i - off) % nsl;
  dst[i] = w_of((long long)b * r, N);
}

cudaError_t stockham_twiddle_fill(float2* dst, int N, int R, cudaStream_t s) {
  const int size = stockham_table_size(N, R);
  if (size <= 0) return cudaSuccess;
  k_stockham_twiddle<<<(size + 255) / 256, 256, 0, s>>>(dst, N, R, size);
  return cudaGetLastError();
}

// dst[m*N1 + n1] = W_N^((n1*m*T) mod N).
__global__ void k_passa_twiddle(float2* dst, int N1, int R, long long T, long long N) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N1 * R) return;
  const long long m = i / N1, n1 = i % N1;
  dst[i] = w_of((n1 * m * T) % N, N);
}

cudaError_t passa_twiddle_fill(float2* dst, int N1, int R, long long T, long long N, cudaStream_t s) {
  k_passa_twiddle<<<(N1 * R + 255) / 256, 256, 0, s>>>(dst, N1, R, T, N);
  return cudaGetLastError();
}

// 4-bit complex expansion (bit-exact replacement of the reference's LUT
// kernels complex4_expansion / copy_expand_complex4, rawspec_gpu.cu:342-374):
// packed byte b -> real = sign-extended high nibble, imag = sign-extended low
// nibble.  The packed staging buffer already has the reference's corner-turned
// layout [channel][block][time][pol], so the expansion is a pure stream.
__device__ __forceinline__ uint32_t expand2(uint32_t b0, uint32_t b1) {
  // two packed bytes -> four int8 components (re0, im0, re1, im1)
  const uint32_t r0 = (uint32_t)(uint8_t)((int8_t)(b0 & 0xf0) >> 4);
  const uint32_t i0 = (uint32_t)(uint8_t)((int8_t)(b0 << 4) >> 4);
  const uint32_t r1 = (uint32_t)(uint8_t)((int8_t)(b1 & 0xf0) >> 4);
  const uint32_t i1 = (uint32_t)(uint8_t)((int8_t)(b1 << 4) >> 4);
  return r0 | (i0 << 8) | (r1 << 16) | (i1 << 24);
}

// Four packed bytes -> eight int8 components (re, im, re, im, ...): both
// nibbles of every byte at once, sign-extended as (x ^ 8) - 8 per byte, then
// interleaved high (real) / low (imaginary).
__device__ __forceinline__ uint2 expand_word(uint32_t w) {
  const uint32_t hi = __vsub4(((w >> 4) & 0x0f0f0f0fu) ^ 0x08080808u, 0x08080808u);
  const uint32_t lo = __vsub4((w & 0x0f0f0f0fu) ^ 0x08080808u, 0x08080808u);
  return make_uint2(__byte_perm(hi, lo, 0x5140), __byte_perm(hi, lo, 0x7362));
}

// 16 packed bytes per thread; grid.y = (block, channel) segments of the
// launch, grid.x covers one segment (blk_bytes_packed % 16 == 0).
__global__ void k_expand4_vec(Expand4Launch a) {
  const int seg = blockIdx.y;
  const int c = a.c0 + seg % a.nch;
  const int blk = (a.dst_block + seg / a.nch) % a.Nb;
  const long long pin = (long long)c * a.Nb * a.blk_bytes_packed + (long long)blk * a.blk_bytes_packed;
  const long long n16 = a.blk_bytes_packed / 16;
  const uint4* src = reinterpret_cast<const uint4*>(a.packed + pin);
  uint4* dst = reinterpret_cast<uint4*>(a.out + 2 * pin);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n16; i += (long long)gridDim.x * blockDim.x) {
    const uint4 p = __ldg(src + i);
    const uint2 e0 = expand_word(p.x), e1 = expand_word(p.y), e2 = expand_word(p.z), e3 = expand_word(p.w);
    dst[2 * i] = make_uint4(e0.x, e0.y, e1.x, e1.y);
    dst[2 * i + 1] = make_uint4(e2.x, e2.y, e3.x, e3.y);
  }
}

__global__ void k_expand4_words(Expand4Launch a) {
  // one thread per 4 packed bytes; blk_bytes_packed % 4 == 0
  const long long words_per_seg = a.blk_bytes_packed / 4;
  const long long total = words_per_seg * a.nch * a.num_blocks;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long w = i % words_per_seg;
    const long long seg = i / words_per_seg;
    const int c = a.c0 + (int)(seg % a.nch);
    const int bi = (int)(seg / a.nch);
    const int blk = (a.dst_block + bi) % a.Nb;
    const long long pin = (long long)c * a.Nb * a.blk_bytes_packed + (long long)blk * a.blk_bytes_packed;
    const uint32_t p = *reinterpret_cast<const uint32_t*>(a.packed + pin + 4 * w);
    uint2 o;
    o.x = expand2(p & 0xff, (p >> 8) & 0xff);
    o.y = expand2((p >> 16) & 0xff, p >> 24);
    *reinterpret_cast<uint2*>(a.out + 2 * pin + 8 * w) = o;
  }
}

__global__ void k_expand4_bytes(Expand4Launch a) {
  const long long total = a.blk_bytes_packed * a.nch * a.num_blocks;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long b = i % a.blk_bytes_packed;
    const long long seg = i / a.blk_bytes_packed;
    const int c = a.c0 + (int)(seg % a.nch);
    const int bi = (int)(seg / a.nch);
    const int blk = (a.dst_block + bi) % a.Nb;
    const long long pin = (long long)c * a.Nb * a.blk_bytes_packed + (long long)blk * a.blk_bytes_packed + b;
    const uint8_t v = a.packed[pin];
    a.out[2 * pin] = (int8_t)(v & 0xf0) >> 4;
    a.out[2 * pin + 1] = (int8_t)(uint8_t)(v << 4) >> 4;
  }
}

cudaError_t expand4_launch(const Expand4Launch& Lin, cudaStream_t s) {
  Expand4Launch L = Lin;
  if (L.nch < 0) {
    L.c0 = 0;
    L.nch = L.Nc;
  }
  const long long nseg = (long long)L.nch * L.num_blocks;
  if (L.blk_bytes_packed % 16 == 0 && nseg >= 1 && nseg <= 65535 &&
      (reinterpret_cast<uintptr_t>(L.packed) & 15) == 0 && (reinterpret_cast<uintptr_t>(L.out) & 15) == 0) {
    const long long n16 = L.blk_bytes_packed / 16;
    const long long want = std::max<long long>(1, (152LL * 16 + nseg - 1) / nseg);  // ~16 CTAs per SM in all
    const int gx = (int)std::max<long long>(1, std::min<long long>((n16 + 255) / 256, want));
    k_expand4_vec<<<dim3(gx, (unsigned)nseg), 256, 0, s>>>(L);
    return cudaGetLastError();
  }
  const bool words = (L.blk_bytes_packed % 4) == 0;
  const long long items = (words ? L.blk_bytes_packed / 4 : L.blk_bytes_packed) * L.nch * L.num_blocks;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((items + 255) / 256, 152LL * 32));
  if (words) k_expand4_words<<<blocks, 256, 0, s>>>(L);
  else k_expand4_bytes<<<blocks, 256, 0, s>>>(L);
  return cudaGetLastError();
}

// Weighted incoherent sum over antennas (the reference's incoherent_sum,
// rawspec_gpu.cu:321-340): ics = sum_a w[a] * P[antenna a], accumulated in
// antenna order with fused multiply-adds from zero.  Both buffers are already
// FFT-shifted, so the fine-channel index maps straight through.
__global__ void k_ics(IcsLaunch a) {
  const int Nca = a.Nc / a.Nant;
  const long long per_plane = (long long)Nca * a.N;
  const long long total = (long long)a.Nd * a.np * per_plane;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const long long within = i % per_plane;   // c*N + f
    const long long dp = i / per_plane;       // d*np + p
    const float* src = a.pwr + dp * (long long)a.Nc * a.N + within;
    float s = 0.0f;
    for (int ant = 0; ant < a.Nant; ++ant) s = __fmaf_rn(a.w[ant], src[(long long)ant * per_plane], s);
    a.ics[i] = s;
  }
}

cudaError_t ics_launch(const IcsLaunch& L, cudaStream_t s) {
  const long long total = (long long)L.Nd * L.np * (L.Nc / L.Nant) * L.N;
  const int blocks = (int)std::max<long long>(1, std::min<long long>((total + 255) / 256, 152LL * 16));
  k_ics<<<blocks, 256, 0, s>>>(L);
  return cudaGetLastError();
}

// One step of compensated summation (Kahan, "Further remarks on reducing
// truncation errors", CACM 8(1), 1965): the low-order part lost when x is
// added to s is carried in c and taken off the next term.  Round-to-nearest
// intrinsics keep the compiler from contracting or reassociating the four
// operations.
__device__ __forceinline__ void kahan_step(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}

// Streams the three planes once: 16-byte accesses over the first n4 groups
// of four floats, single floats over the tail.
__global__ void k_kahan_merge(float* __restrict__ sum, float* __restrict__ comp, const float* __restrict__ stage,
                              long long n, long long n4) {
  const long long stride = (long long)gridDim.x * blockDim.x;
  const long long i0 = blockIdx.x * (long long)blockDim.x + threadIdx.x;
  float4* s4 = reinterpret_cast<float4*>(sum);
  float4* c4 = reinterpret_cast<float4*>(comp);
  const float4* x4 = reinterpret_cast<const float4*>(stage);
  for (long long i = i0; i < n4; i += stride) {
    float4 s = s4[i], c = c4[i];
    const float4 x = __ldcs(x4 + i);
    kahan_step(s.x, c.x, x.x);
    kahan_step(s.y, c.y, x.y);
    kahan_step(s.z, c.z, x.z);
    kahan_step(s.w, c.w, x.w);
    s4[i] = s;
    c4[i] = c;
  }
  for (long long i = 4 * n4 + i0; i < n; i += stride) {
    float s = sum[i], c = comp[i];
    kahan_step(s, c, __ldcs(stage + i));
    sum[i] = s;
    comp[i] = c;
  }
}

cudaError_t kahan_merge_launch(float* sum, float* comp, const float* stage, long long n, cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  const bool vec = ((reinterpret_cast<uintptr_t>(sum) | reinterpret_cast<uintptr_t>(comp) |
                     reinterpret_cast<uintptr_t>(stage)) & 15) == 0;
  const long long n4 = vec ? n / 4 : 0;
  const long long items = std::max(n4, n - 4 * n4);
  const int blocks = (int)std::max<long long>(1, std::min<long long>((items + 255) / 256, 152LL * 8));
  k_kahan_merge<<<blocks, 256, 0, s>>>(sum, comp, stage, n, n4);
  return cudaGetLastError();
}

}  // namespace rsg
