// common.cuh -- shared device helpers for the GB300 spectrometer kernels.
//
// Sample formats, the integer -> float conversion of the GUPPI voltages and
// small complex helpers.  Everything here is header-only device code that is
// inlined into the kernels of k_small.cu, k_large.cu and k_aux.cu.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

#include "internal.h"

namespace rsg {

// ----------------------------------------------------------------------------
// Sample formats of the device input buffer.  The device buffer is laid out
// [channel][time][pol][re,im] with the Nb blocks of a buffer concatenated per
// channel (the corner turn done by the host->device copy), exactly the order
// the reference gives its FFT input (rawspec_gpu.cu:1454-1460).
// ----------------------------------------------------------------------------

// Integer -> float conversion of one component as the reference performs it.
// The reference reads the input through a CUDA texture in
// cudaReadModeNormalizedFloat (rawspec_gpu.cu:133-148, :845-866), which maps a
// signed n-bit code x to x / (2^(n-1) - 1), clamped to -1.0 for the most
// negative code.  snorm() computes the correctly rounded quotient with one
// multiply and one FMA-based correction step, which is exact for every 8- and
// 16-bit code (checked exhaustively) and matches the texture unit bit for bit
// (GPU probe test).  The kernels use the equivalent integer form below.
template <int D>
__device__ __forceinline__ float snorm(int x) {
  constexpr float d = (float)D;
  constexpr float r = 1.0f / (float)D;
  x = x < -D ? -D : x;
  const float f = (float)x;
  float q = f * r;
  const float e = __fmaf_rn(-q, d, f);
  return __fmaf_rn(e, r, q);
}

// Word type holding one time sample (all polarisations) of a format.
template <int FMT, int NP> struct SampleWord;
template <> struct SampleWord<FMT_I8, 2> { using type = uint32_t; };
template <> struct SampleWord<FMT_I8, 1> { using type = uint16_t; };
template <> struct SampleWord<FMT_I16, 2> { using type = uint2; };
template <> struct SampleWord<FMT_I16, 1> { using type = uint32_t; };

// Integer unpack used by the kernels: the exact integer codes as floats, with
// the most negative code clamped like the texture's SNORM mapping (-128 ->
// -127, -32768 -> -32767) and the 1/127 (1/32767) SNORM scale left out.
// Every detected product is quadratic in the samples, so the kernels apply
// the scale once, as 1/127^2 (1/32767^2), to the integrated results.  The
// codes themselves (and the 4-bit nibble expansion) are bit-exact.
__device__ __forceinline__ void unpack_word_int(uint32_t w, float2 (&o)[2]) {
  w = __vmaxs4(w, 0x81818181u);
  o[0] = make_float2((float)(int8_t)(w & 0xff), (float)(int8_t)((w >> 8) & 0xff));
  o[1] = make_float2((float)(int8_t)((w >> 16) & 0xff), (float)(int8_t)(w >> 24));
}
__device__ __forceinline__ void unpack_word_int(uint16_t w16, float2 (&o)[1]) {
  const uint32_t w = __vmaxs4((uint32_t)w16, 0x81818181u);
  o[0] = make_float2((float)(int8_t)(w & 0xff), (float)(int8_t)((w >> 8) & 0xff));
}
__device__ __forceinline__ void unpack_word_int(uint2 w, float2 (&o)[2]) {
  const uint32_t a = __vmaxs2(w.x, 0x80018001u), b = __vmaxs2(w.y, 0x80018001u);
  o[0] = make_float2((float)(int16_t)(a & 0xffff), (float)(int16_t)(a >> 16));
  o[1] = make_float2((float)(int16_t)(b & 0xffff), (float)(int16_t)(b >> 16));
}
__device__ __forceinline__ void unpack_word_int(uint32_t w, float2 (&o)[1], int /*int16 tag*/) {
  const uint32_t a = __vmaxs2(w, 0x80018001u);
  o[0] = make_float2((float)(int16_t)(a & 0xffff), (float)(int16_t)(a >> 16));
}

// Loads-and-unpacks one sample word of format FMT with NP polarisations.
template <int FMT, int NP>
struct Unpack;
template <> struct Unpack<FMT_I8, 2> {
  static __device__ __forceinline__ void run(uint32_t w, float2 (&o)[2]) { unpack_word_int(w, o); }
};
template <> struct Unpack<FMT_I8, 1> {
  static __device__ __forceinline__ void run(uint16_t w, float2 (&o)[1]) { unpack_word_int(w, o); }
};
template <> struct Unpack<FMT_I16, 2> {
  static __device__ __forceinline__ void run(uint2 w, float2 (&o)[2]) { unpack_word_int(w, o); }
};
template <> struct Unpack<FMT_I16, 1> {
  static __device__ __forceinline__ void run(uint32_t w, float2 (&o)[1]) { unpack_word_int(w, o, 16); }
};

// ----------------------------------------------------------------------------
// Complex helpers.
// ----------------------------------------------------------------------------
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }
// a * w
__device__ __forceinline__ float2 cmul(float2 a, float2 w) {
  return make_float2(__fmaf_rn(a.x, w.x, -a.y * w.y), __fmaf_rn(a.x, w.y, a.y * w.x));
}

// cos(pi t / 16) for t in [0, 16], as decimal literals (non-recursive, so a
// constant argument always folds).
__host__ __device__ constexpr double cos_pi16(int t) {
  return t == 0 ? 1.0
       : t == 1 ? 0.98078528040323043
       : t == 2 ? 0.92387953251128674
       : t == 3 ? 0.83146961230254524
       : t == 4 ? 0.70710678118654757
       : t == 5 ? 0.55557023301960229
       : t == 6 ? 0.38268343236508984
       : t == 7 ? 0.19509032201612833
       : t == 8 ? 0.0
       : t == 9 ? -0.19509032201612833
       : t == 10 ? -0.38268343236508984
       : t == 11 ? -0.55557023301960229
       : t == 12 ? -0.70710678118654757
       : t == 13 ? -0.83146961230254524
       : t == 14 ? -0.92387953251128674
       : t == 15 ? -0.98078528040323043
       : -1.0;
}
// sin(pi t / 16) for t in [0, 16).
__host__ __device__ constexpr double sin_pi16(int t) {
  return t <= 8 ? cos_pi16(8 - t) : cos_pi16(t - 8);
}

// Multiply a by the forward twiddle exp(-2 pi i k / len) for 0 <= k < len/2,
// len a power of two <= 32.  After loop unrolling k and len are constants, so
// the trivial cases cost no multiplies.
__device__ __forceinline__ float2 twiddle_fwd(float2 a, int k, int len) {
  if (k == 0) return a;
  const int t = (32 / len) * k;  // angle = pi t / 16
  if (t == 8) return make_float2(a.y, -a.x);  // * (-i)
  if (t == 4) {                               // * (1 - i)/sqrt(2)
    constexpr float h = 0.70710678118654752f;
    return make_float2((a.x + a.y) * h, (a.y - a.x) * h);
  }
  if (t == 12) {                              // * (-1 - i)/sqrt(2)
    constexpr float h = 0.70710678118654752f;
    return make_float2((a.y - a.x) * h, -(a.x + a.y) * h);
  }
  const float c = (float)cos_pi16(t);
  const float s = (float)sin_pi16(t);
  // (a.x + i a.y)(c - i s)
  return make_float2(__fmaf_rn(a.x, c, a.y * s), __fmaf_rn(a.y, c, -a.x * s));
}

}  // namespace rsg
