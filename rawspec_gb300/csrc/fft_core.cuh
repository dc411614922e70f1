// fft_core.cuh -- the FFT engine of the spectrometer kernels.
//
// Two levels:
//   * dft_regs<R>: an R-point DFT (R a power of two <= 32) held entirely in
//     registers; radix-2 decimation in frequency with compile-time twiddles,
//     natural order in and out.
//   * GroupFFT<N, R, NV>: an N-point FFT computed by a group of T = N/R
//     threads, each holding R values of NV independent vectors (the two
//     polarisations share every twiddle).  Stockham auto-sort passes of radix
//     R (a smaller radix for the last pass when N is not a power of R), with
//     one shared-memory exchange between passes.  On entry thread j holds
//     x[j + m*T] in v[.][m]; on exit it holds X[j + m*T].  The formulation is
//     the classic per-thread Stockham iteration (Govindaraju et al., SC08).
//
// All FFTs here are forward, exp(-2 pi i k n / N), unnormalised; the inverse
// transform is obtained by the index reversal X_inv[k] = X_fwd[(N-k) mod N]
// applied where results are stored.
//
// Two vectors in lockstep (NV = 2, the two polarisations) run on the packed
// FP32 instructions of sm_100 and later (add/sub/mul/fma .f32x2, each lane
// rounded exactly as the scalar _rn operation): element m of both vectors is
// held as a cpair {re: (x0.re, x1.re), im: (x0.im, x1.im)}, so that one
// instruction does the work of two, with the twiddles shared by both lanes.
// RSG_PACKED=0 selects the scalar form.
#pragma once

#include "common.cuh"

#ifndef RSG_PACKED
#define RSG_PACKED 1
#endif

namespace rsg {

// ---- packed pairs -----------------------------------------------------------
struct cpair {
  float2 re, im;  // lane 0: vector 0, lane 1: vector 1
};

__device__ __forceinline__ float2 f2add(float2 a, float2 b) { return __fadd2_rn(a, b); }
__device__ __forceinline__ float2 f2mul(float2 a, float2 b) { return __fmul2_rn(a, b); }
__device__ __forceinline__ float2 f2fma(float2 a, float2 b, float2 c) { return __ffma2_rn(a, b, c); }
__device__ __forceinline__ float2 f2sub(float2 a, float2 b) {
  float2 r;
  asm("{\n\t.reg .b64 ra, rb, rr;\n\t"
      "mov.b64 ra, {%2, %3};\n\t"
      "mov.b64 rb, {%4, %5};\n\t"
      "sub.rn.f32x2 rr, ra, rb;\n\t"
      "mov.b64 {%0, %1}, rr;\n\t}"
      : "=f"(r.x), "=f"(r.y)
      : "f"(a.x), "f"(a.y), "f"(b.x), "f"(b.y));
  return r;
}
__device__ __forceinline__ float2 f2dup(float x) { return make_float2(x, x); }

__device__ __forceinline__ cpair padd(const cpair& a, const cpair& b) { return {f2add(a.re, b.re), f2add(a.im, b.im)}; }
__device__ __forceinline__ cpair psub(const cpair& a, const cpair& b) { return {f2sub(a.re, b.re), f2sub(a.im, b.im)}; }
// a * w for one twiddle w shared by both lanes
__device__ __forceinline__ cpair pmul(const cpair& a, float2 w) {
  const float2 c = f2dup(w.x), s = f2dup(w.y), ns = f2dup(-w.y);
  return {f2fma(a.im, ns, f2mul(a.re, c)), f2fma(a.re, s, f2mul(a.im, c))};
}
__device__ __forceinline__ cpair pack2(float2 x0, float2 x1) { return {make_float2(x0.x, x1.x), make_float2(x0.y, x1.y)}; }
__device__ __forceinline__ float2 lane0(const cpair& p) { return make_float2(p.re.x, p.im.x); }
__device__ __forceinline__ float2 lane1(const cpair& p) { return make_float2(p.re.y, p.im.y); }

// (a - b) * exp(-2 pi i k / len), 0 <= k < len/2, len a power of two <= 32;
// k and len are compile-time constants after unrolling.
__device__ __forceinline__ cpair pbfly_lo(const cpair& a, const cpair& b, int k, int len) {
  if (k == 0) return psub(a, b);
  const int t = (32 / len) * k;  // angle = pi t / 16
  if (t == 8) return {f2sub(a.im, b.im), f2sub(b.re, a.re)};  // * (-i)
  const cpair d = psub(a, b);
  constexpr float h = 0.70710678118654752f;
  if (t == 4) return {f2mul(f2add(d.re, d.im), f2dup(h)), f2mul(f2sub(d.im, d.re), f2dup(h))};
  if (t == 12) return {f2mul(f2sub(d.im, d.re), f2dup(h)), f2mul(f2add(d.re, d.im), f2dup(-h))};
  const float c = (float)cos_pi16(t);
  const float s = (float)sin_pi16(t);
  // (x + i y)(c - i s) = (x c + y s) + i (y c - x s)
  return {f2fma(d.im, f2dup(s), f2mul(d.re, f2dup(c))), f2fma(d.re, f2dup(-s), f2mul(d.im, f2dup(c)))};
}

__host__ __device__ constexpr int ilog2(int n) { return n <= 1 ? 0 : 1 + ilog2(n >> 1); }
__host__ __device__ constexpr int bitrev(int x, int bits) {
  return bits == 0 ? 0 : ((x & 1) << (bits - 1)) | bitrev(x >> 1, bits - 1);
}

// Compile-time bit-reversal permutation of a register array.
template <int R, int M>
struct BitrevSwap {
  static __device__ __forceinline__ void apply(float2 (&v)[R]) {
    constexpr int BR = bitrev(M, ilog2(R));
    if constexpr (M < BR) {
      const float2 t = v[M];
      v[M] = v[BR];
      v[BR] = t;
    }
    BitrevSwap<R, M + 1>::apply(v);
  }
};
template <int R>
struct BitrevSwap<R, R> {
  static __device__ __forceinline__ void apply(float2 (&)[R]) {}
};

// In-register DFT of R points (R = 1, 2, 4, 8, 16, 32), natural order.
template <int R>
__device__ __forceinline__ void dft_regs(float2 (&v)[R]) {
  if constexpr (R > 1) {
#pragma unroll
    for (int len = R; len >= 2; len >>= 1) {
      const int half = len >> 1;
#pragma unroll
      for (int i = 0; i < R; i += len) {
#pragma unroll
        for (int k = 0; k < half; ++k) {
          const float2 a = v[i + k];
          const float2 b = v[i + k + half];
          v[i + k] = cadd(a, b);
          v[i + k + half] = twiddle_fwd(csub(a, b), k, len);
        }
      }
    }
    // Outputs are in bit-reversed order: undo with compile-time swaps.
    BitrevSwap<R, 0>::apply(v);
  }
}

template <int R, int M>
struct BitrevSwapP {
  static __device__ __forceinline__ void apply(cpair (&v)[R]) {
    constexpr int BR = bitrev(M, ilog2(R));
    if constexpr (M < BR) {
      const cpair t = v[M];
      v[M] = v[BR];
      v[BR] = t;
    }
    BitrevSwapP<R, M + 1>::apply(v);
  }
};
template <int R>
struct BitrevSwapP<R, R> {
  static __device__ __forceinline__ void apply(cpair (&)[R]) {}
};

// dft_regs on packed pairs.
template <int R>
__device__ __forceinline__ void dft_regs2(cpair (&v)[R]) {
  if constexpr (R > 1) {
#pragma unroll
    for (int len = R; len >= 2; len >>= 1) {
      const int half = len >> 1;
#pragma unroll
      for (int i = 0; i < R; i += len) {
#pragma unroll
        for (int k = 0; k < half; ++k) {
          const cpair a = v[i + k];
          const cpair b = v[i + k + half];
          v[i + k] = padd(a, b);
          v[i + k + half] = pbfly_lo(a, b, k, len);
        }
      }
    }
    BitrevSwapP<R, 0>::apply(v);
  }
}

template <int RP, int STRIDE, int R>
__device__ __forceinline__ void dft_subset2(cpair (&v)[R], int off) {
  cpair t[RP];
#pragma unroll
  for (int s = 0; s < RP; ++s) t[s] = v[off + s * STRIDE];
  dft_regs2<RP>(t);
#pragma unroll
  for (int s = 0; s < RP; ++s) v[off + s * STRIDE] = t[s];
}

// DFT over a strided subset of a register array: elements v[off + s*STRIDE],
// s = 0..RP-1, with RP*STRIDE <= R.
template <int RP, int STRIDE, int R>
__device__ __forceinline__ void dft_subset(float2 (&v)[R], int off) {
  float2 t[RP];
#pragma unroll
  for (int s = 0; s < RP; ++s) t[s] = v[off + s * STRIDE];
  dft_regs<RP>(t);
#pragma unroll
  for (int s = 0; s < RP; ++s) v[off + s * STRIDE] = t[s];
}

// Shared-memory index with a padding word every 16 complex values, which
// keeps the strided writes of the Stockham passes free of bank conflicts:
// element e lives at e + (e >> 4).  GroupFFT computes these positions as a
// per-thread base plus compile-time offsets, which is exact because every
// pass's write stride Ns*R and read stride T are powers of two.
__device__ __forceinline__ int smem_pad(int e) { return e + (e >> 4); }
__host__ __device__ constexpr int smem_padded_len(int n) { return n + (n >> 4) + 1; }

// Number of radix-R passes and the radix of the trailing pass.
template <int N, int R>
struct FftShape {
  static constexpr int T = N / R;                       // threads per FFT
  static constexpr int LOGN = ilog2(N);
  static constexpr int LOGR = ilog2(R);
  static constexpr int FULL = (LOGR == 0) ? 0 : LOGN / LOGR;     // radix-R passes
  static constexpr int RLAST = (LOGR == 0) ? 1 : (1 << (LOGN - FULL * LOGR));
  static constexpr int PASSES = FULL + (RLAST > 1 ? 1 : 0);
};

// Twiddle table of a GroupFFT<N, R>, one block per twiddled pass, laid out so
// that the lanes of a warp read consecutive (or identical) entries:
//   full pass p >= 1 (Ns = R^p):    [r-1][k]  = W_N^(k r N/(Ns R)), k < Ns
//   trailing pass (radix RL):       [r-1][b]  = W_N^(b r),          b < N/RL
// StockhamTw<N, R>::offset(p) is the start of pass p's block; `size` the total.
__host__ __device__ constexpr int stockham_tw_offset(int N, int R, int p) {
  // blocks of passes 1 .. p-1
  int off = 0, Ns = R;
  for (int q = 1; q < p; ++q) {
    off += (R - 1) * Ns;
    Ns *= R;
  }
  return off;
}
__host__ __device__ constexpr int stockham_tw_size(int N, int R) {
  if (R <= 1 || N <= R) return 0;
  int full = 0, Ns = 1;
  while (Ns * R <= N) {
    Ns *= R;
    ++full;
  }
  const int rl = N / Ns;
  return stockham_tw_offset(N, R, full) + (rl > 1 ? (rl - 1) * (N / rl) : 0);
}

// Group FFT.  tw: the pass-ordered twiddle table described above (shared or
// global memory).  sm: this group's exchange buffers, NV buffers of
// smem_padded_len(N) float2 each, spaced by `sm_stride` float2.  SYNC is a
// functor performing the barrier required between the group's threads.
template <int N, int R, int NV>
struct GroupFFT {
  using S = FftShape<N, R>;
  static constexpr int T = S::T;

  template <typename Sync>
  static __device__ __forceinline__ void run(float2 (&v)[NV][R], int j, float2* sm, int sm_stride,
                                             const float2* __restrict__ tw, Sync sync) {
    if constexpr (NV == 2 && RSG_PACKED) {
      cpair p[R];
#pragma unroll
      for (int m = 0; m < R; ++m) p[m] = pack2(v[0][m], v[1][m]);
      run_packed(p, j, sm, sm_stride, tw, sync);
#pragma unroll
      for (int m = 0; m < R; ++m) {
        v[0][m] = lane0(p[m]);
        v[1][m] = lane1(p[m]);
      }
    } else {
      run_scalar(v, j, sm, sm_stride, tw, sync);
    }
  }

  // Both vectors as packed pairs; the exchange buffers hold the re pairs
  // (first buffer) and the im pairs (second buffer) at the positions the
  // scalar form gives the two vectors' values.  SPLIT: one exchange buffer
  // only (sm_stride unused), the re pairs and then the im pairs passing
  // through it (twice the barriers, half the shared memory).
  template <bool SPLIT = false, typename Sync>
  static __device__ __forceinline__ void run_packed(cpair (&v)[R], int j, float2* sm, int sm_stride,
                                                    const float2* __restrict__ tw, Sync sync) {
    if constexpr (T == 1) {
      dft_regs2<R>(v);
    } else {
      int Ns = 1;
#pragma unroll
      for (int p = 0; p < S::FULL; ++p) {
        if (p > 0) {
          const int k = j & (Ns - 1);
          const float2* twp = tw + stockham_tw_offset(N, R, p) + k;
#pragma unroll
          for (int r = 1; r < R; ++r) v[r] = pmul(v[r], twp[(r - 1) * Ns]);
        }
        dft_regs2<R>(v);
        const bool last = (p == S::FULL - 1) && (S::RLAST == 1);
        if (!last) {
          const int lo = j & (Ns - 1);
          const int hi = j / Ns;
          const int idxD = hi * Ns * R + lo;
          const int wbase = idxD + ((hi * Ns * R) >> 4) + (Ns >= 16 ? (lo >> 4) : 0);
          const int rbase = j + (T >= 16 ? (j >> 4) : 0);
          if constexpr (SPLIT) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
#pragma unroll
              for (int r = 0; r < R; ++r) {
                const int off = Ns >= 16 ? r * (Ns + (Ns >> 4)) : r * Ns + ((r * Ns) >> 4);
                sm[wbase + off] = h == 0 ? v[r].re : v[r].im;
              }
              sync();
#pragma unroll
              for (int m = 0; m < R; ++m) {
                const int off = T >= 16 ? m * (T + (T >> 4)) : m * T + ((m * T) >> 4);
                if (h == 0) v[m].re = sm[rbase + off]; else v[m].im = sm[rbase + off];
              }
              sync();
            }
          } else {
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const int off = Ns >= 16 ? r * (Ns + (Ns >> 4)) : r * Ns + ((r * Ns) >> 4);
              sm[wbase + off] = v[r].re;
              sm[sm_stride + wbase + off] = v[r].im;
            }
            sync();
#pragma unroll
            for (int m = 0; m < R; ++m) {
              const int off = T >= 16 ? m * (T + (T >> 4)) : m * T + ((m * T) >> 4);
              v[m].re = sm[rbase + off];
              v[m].im = sm[sm_stride + rbase + off];
            }
            sync();
          }
        }
        Ns *= R;
      }
      if constexpr (S::RLAST > 1) {
        constexpr int RL = S::RLAST;
        constexpr int Q = R / RL;
        constexpr int NSL = N / RL;
        const float2* twl = tw + stockham_tw_offset(N, R, S::FULL) + j;
#pragma unroll
        for (int qb = 0; qb < Q; ++qb) {
#pragma unroll
          for (int r = 1; r < RL; ++r) v[qb + r * Q] = pmul(v[qb + r * Q], twl[(r - 1) * NSL + qb * T]);
          dft_subset2<RL, Q>(v, qb);
        }
      }
    }
  }

  template <typename Sync>
  static __device__ __forceinline__ void run_scalar(float2 (&v)[NV][R], int j, float2* sm, int sm_stride,
                                                    const float2* __restrict__ tw, Sync sync) {
    if constexpr (T == 1) {
      // One thread holds the whole transform.
#pragma unroll
      for (int q = 0; q < NV; ++q) dft_regs<R>(v[q]);
    } else {
      int Ns = 1;
#pragma unroll
      for (int p = 0; p < S::FULL; ++p) {
        // Twiddles (identity on the first pass).
        if (p > 0) {
          const int k = j & (Ns - 1);
          const float2* twp = tw + stockham_tw_offset(N, R, p) + k;
#pragma unroll
          for (int r = 1; r < R; ++r) {
            const float2 w = twp[(r - 1) * Ns];
#pragma unroll
            for (int q = 0; q < NV; ++q) v[q][r] = cmul(v[q][r], w);
          }
        }
#pragma unroll
        for (int q = 0; q < NV; ++q) dft_regs<R>(v[q]);
        const bool last = (p == S::FULL - 1) && (S::RLAST == 1);
        if (!last) {
          // Padded write positions idxD + r*Ns as a runtime base plus a
          // compile-time offset per r (see smem_pad).
          const int lo = j & (Ns - 1);
          const int hi = j / Ns;
          const int idxD = hi * Ns * R + lo;
          const int wbase = idxD + ((hi * Ns * R) >> 4) + (Ns >= 16 ? (lo >> 4) : 0);
#pragma unroll
          for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int r = 0; r < R; ++r) {
              const int off = Ns >= 16 ? r * (Ns + (Ns >> 4)) : r * Ns + ((r * Ns) >> 4);
              sm[q * sm_stride + wbase + off] = v[q][r];
            }
          sync();
          const int rbase = j + (T >= 16 ? (j >> 4) : 0);
#pragma unroll
          for (int q = 0; q < NV; ++q)
#pragma unroll
            for (int m = 0; m < R; ++m) {
              const int off = T >= 16 ? m * (T + (T >> 4)) : m * T + ((m * T) >> 4);
              v[q][m] = sm[q * sm_stride + rbase + off];
            }
          sync();
        }
        Ns *= R;
      }
      if constexpr (S::RLAST > 1) {
        // Trailing pass of radix RL < R: thread j computes Q = R/RL
        // butterflies b = j + q*T on elements m = q + r*Q.
        constexpr int RL = S::RLAST;
        constexpr int Q = R / RL;
        constexpr int NSL = N / RL;
        const float2* twl = tw + stockham_tw_offset(N, R, S::FULL) + j;
#pragma unroll
        for (int qb = 0; qb < Q; ++qb) {
          // butterfly b = j + qb*T; its twiddles W_N^(b r) sit at [r-1][b]
#pragma unroll
          for (int r = 1; r < RL; ++r) {
            const float2 w = twl[(r - 1) * NSL + qb * T];
#pragma unroll
            for (int q = 0; q < NV; ++q) v[q][qb + r * Q] = cmul(v[q][qb + r * Q], w);
          }
#pragma unroll
          for (int q = 0; q < NV; ++q) dft_subset<RL, Q>(v[q], qb);
        }
      }
    }
  }
};

}  // namespace rsg
