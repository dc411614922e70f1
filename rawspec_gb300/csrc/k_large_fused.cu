// k_large_fused.cu -- persistent four-step FFT spectrometer for long
// transforms whose integration unit is one spectrum per buffer (the case of
// the 2^20-point product of the production configuration).
//
// The two passes of the four-step FFT (see k_large.cu) become work items of
// one persistent kernel, taken in a fixed order through an atomic counter
// (here with a lag of 2):
//
//   A(0) A(1) A(2) B(0) A(3) B(1) ... A(S-1) B(S-3) B(S-2) B(S-1)
//
// where A(s) are the column tiles of slab s (one channel-spectrum, both
// polarisations) and B(s) its row tiles.  A(s) writes the FP32 intermediate
// into slot s mod RING of a small ring (RING slabs, sized to stay in L2);
// B(s) waits until every A(s) tile is published, A(s) waits until every
// B(s-RING) tile has released the slot.  An item only ever waits for items
// earlier in the order, which were taken by CTAs that are running, so the
// waits always end; they are bounded nonetheless and record an error instead
// of hanging if the bound is ever reached.  Column and row tiles of
// neighbouring slabs run side by side on the SMs, so the loads of one overlap
// the arithmetic of another, and the intermediate rarely leaves L2.
#include <algorithm>

#include "detect.cuh"
#include "fft_core.cuh"
#include "internal.h"

namespace rsg {

namespace {

constexpr int kFusedTPB = 256;
#ifndef RSG_FUSED_LAG
#define RSG_FUSED_LAG 2
#endif
#ifndef RSG_FUSED_RING
#define RSG_FUSED_RING 4
#endif
// Row tiles of slab s are queued after the column tiles of slab s + kLag, so
// that a row tile rarely finds its slab's column tiles still running; a slot
// of the intermediate ring is reused kRingSlots slabs later (> kLag keeps
// every wait pointed at earlier items).
constexpr int kLag = RSG_FUSED_LAG;
constexpr int kRingSlots = RSG_FUSED_RING;
static_assert(kRingSlots > kLag, "a slot must be released by row tiles queued before its next column tiles");
#ifndef RSG_FUSED_K
#define RSG_FUSED_K 2
#endif
constexpr int kTilesPerItem = RSG_FUSED_K;  // tiles per work item (amortises the item overheads)
constexpr long long kSpinLimit = 1ll << 24;  // ~2 s of polling at most

// Radices (values per thread per transform).  Row tiles hold no
// multi-spectrum accumulators (one spectrum per unit); the cross-pol modes
// keep X0 while X1 is transformed, so they stay at 16.
#ifndef RSG_FUSED_RA
#define RSG_FUSED_RA 16
#endif
#ifndef RSG_FUSED_RB_TP
#define RSG_FUSED_RB_TP 16
#endif
__host__ __device__ constexpr int fused_ra() { return RSG_FUSED_RA; }
template <int POL>
__host__ __device__ constexpr int fused_rb() { return POL == POL_TP ? RSG_FUSED_RB_TP : 16; }

// Resident CTAs per SM the register budget is set for: the polarisations are
// transformed one after the other (16 complex values per thread), which
// leaves room for three CTAs in total-power mode; the cross-pol modes keep the
// first polarisation's spectrum while the second is transformed.
#ifndef RSG_FUSED_TP_MINB
#define RSG_FUSED_TP_MINB 2
#endif
template <int POL>
__host__ __device__ constexpr int fused_minb() { return POL == POL_TP ? RSG_FUSED_TP_MINB : 2; }

// Shared-memory distance between the exchange buffers of neighbouring
// interleaved sub-FFTs, chosen so that the C sub-FFTs served by one
// half-warp land on disjoint banks.
__host__ __device__ constexpr int group_stride(int N, int NV, int C) {
  int base = NV * smem_padded_len(N);
  const int cp = C < 16 ? C : 16;
  const int want = (16 / cp) % 16;
  while (base % 16 != want) ++base;
  return base;
}

template <int N1, int N2, int NV, int POL>
struct FusedCfg {
  static constexpr int RA = fused_ra(), TA = N2 / RA, CA = kFusedTPB / TA;
  static constexpr int RB = fused_rb<POL>(), TB = N1 / RB, CB = kFusedTPB / TB;
  static constexpr int TWA = stockham_tw_size(N2, RA), TWB = stockham_tw_size(N1, RB);
  static constexpr int TWA2 = (TWA + 1) & ~1, TWB2 = (TWB + 1) & ~1;
  static constexpr int GSA = group_stride(N2, 1, CA), GSB = group_stride(N1, 1, CB);
  static constexpr int XCH = CA * GSA > CB * GSB ? CA * GSA : CB * GSB;
  static constexpr size_t SMEM = (size_t)(TWA2 + TWB2 + XCH) * sizeof(float2);
  static_assert(TA * CA == kFusedTPB && TB * CB == kFusedTPB, "sub-FFT threads must tile the CTA");
};

struct Sync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

__device__ __forceinline__ int load_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Thread 0 polls until *cnt reaches target (bounded; on time-out it records
// `code` in the error word and lets the CTA proceed), then the CTA proceeds.
__device__ __forceinline__ void wait_count(const int* cnt, int target, int* err, int code) {
  if (threadIdx.x == 0) {
    unsigned ns = 32;
    long long it = 0;
    while (load_acquire(cnt) < target) {
      if (++it > kSpinLimit) {
        atomicExch(err, code);
        break;
      }
      __nanosleep(ns);
      if (ns < 256) ns *= 2;
    }
    __threadfence();
  }
  __syncthreads();
}

// All threads' global writes of the tile become visible, then the tile is
// counted: the CTA barrier orders every thread's writes before thread 0's
// device-scope fence and release of the counter (the same pattern as a grid
// barrier).
__device__ __forceinline__ void publish(int* cnt, int tiles) {
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    atomicAdd(cnt, tiles);
  }
}

// L2 eviction-priority policies: streams read or written once are marked
// evict-first, the ring intermediate (re-read soon) evict-last.
__device__ __forceinline__ unsigned long long policy_evict_first() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ unsigned long long policy_evict_last() {
  unsigned long long p;
  asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
  return p;
}
__device__ __forceinline__ uint32_t ld_u32_hint(const uint32_t* p, unsigned long long pol) {
  uint32_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ uint16_t ld_u16_hint(const uint16_t* p, unsigned long long pol) {
  uint16_t v;
  asm volatile("ld.global.nc.L2::cache_hint.u16 %0, [%1], %2;" : "=h"(v) : "l"(p), "l"(pol));
  return v;
}
__device__ __forceinline__ void st_f2_hint(float2* p, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ float2 ld_f2_hint(const float2* p, unsigned long long pol) {
  float2 v;
  asm volatile("ld.global.cg.L2::cache_hint.v2.f32 {%0, %1}, [%2], %3;" : "=f"(v.x), "=f"(v.y) : "l"(p), "l"(pol)
               : "memory");
  return v;
}
__device__ __forceinline__ float ld_f_hint(const float* p, unsigned long long pol) {
  float v;
  asm volatile("ld.global.cg.L2::cache_hint.f32 %0, [%1], %2;" : "=f"(v) : "l"(p), "l"(pol) : "memory");
  return v;
}
__device__ __forceinline__ void st_f_hint(float* p, float v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}
template <typename W>
struct HintLoad;
template <>
struct HintLoad<uint32_t> {
  static __device__ __forceinline__ uint32_t ld(const uint32_t* p, unsigned long long pol) { return ld_u32_hint(p, pol); }
};
template <>
struct HintLoad<uint16_t> {
  static __device__ __forceinline__ uint16_t ld(const uint16_t* p, unsigned long long pol) { return ld_u16_hint(p, pol); }
};

}  // namespace

template <int N1, int N2, int FMT, int NV, int POL>
__global__ void __launch_bounds__(kFusedTPB, fused_minb<POL>())
k_large_fused(LargeLaunch a) {
  using F = FusedCfg<N1, N2, NV, POL>;
  constexpr int N = N1 * N2;
  constexpr int NP = PolOut<POL>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* twA = reinterpret_cast<float2*>(smem_raw);
  float2* twB = twA + F::TWA2;
  float2* xch = twB + F::TWB2;
  __shared__ long long s_item;

  const int tid = threadIdx.x;
  for (int i = tid; i < F::TWA; i += kFusedTPB) twA[i] = a.twN2[i];
  for (int i = tid; i < F::TWB; i += kFusedTPB) twB[i] = a.twN1[i];
  __syncthreads();

  const int S = a.S;
  constexpr int tilesA = N1 / F::CA, tilesB = N2 / F::CB;
  constexpr int K = kTilesPerItem;
  static_assert(tilesA % K == 0 && tilesB % K == 0, "items must cover whole tiles");
  constexpr int itemsA = tilesA / K, itemsB = tilesB / K;
  const long long total = (long long)S * (itemsA + itemsB);
  int* err = a.ctl;       // sticky error word (never reset by a launch)
  int* next = a.ctl + 1;
  int* doneA = a.ctl + 2;
  int* doneB = a.ctl + 2 + S;
  const float im_sign = a.conj ? -1.0f : 1.0f;
  const unsigned long long pol_first = policy_evict_first();
  const unsigned long long pol_last = policy_evict_last();

  for (;;) {
    if (tid == 0) s_item = (long long)atomicAdd(reinterpret_cast<unsigned int*>(next), 1u);
    __syncthreads();
    const long long item = s_item;
    __syncthreads();
    if (item >= total) break;

    // Decode the item.  Segment k holds A(k) (k < S) followed by B(k - lag)
    // (k >= lag); each item covers K consecutive tiles of one slab.
    bool isA;
    int slab, titem;
    {
      const int p1 = S < kLag ? S : kLag;                 // A-only segments
      const int mid = S > kLag ? S - kLag : 0;            // A+B segments
      const long long n1 = (long long)p1 * itemsA;
      const long long n2 = (long long)mid * (itemsA + itemsB);
      if (item < n1) {
        isA = true;
        slab = (int)(item / itemsA);
        titem = (int)(item % itemsA);
      } else if (item < n1 + n2) {
        const long long i2 = item - n1;
        const int k = kLag + (int)(i2 / (itemsA + itemsB));
        const int r = (int)(i2 % (itemsA + itemsB));
        isA = r < itemsA;
        slab = isA ? k : k - kLag;
        titem = isA ? r : r - itemsA;
      } else {                                            // B-only tail
        const long long i3 = item - n1 - n2;
        isA = false;
        slab = mid + (int)(i3 / itemsB);
        titem = (int)(i3 % itemsB);
      }
    }
    const int slot = slab % a.ring;
    float2* scr = a.scratch + (size_t)slot * NV * N;

    if (isA) {
      if (slab >= a.ring) wait_count(doneB + (slab - a.ring), tilesB, err, 1);
      // ---- K column tiles: N2-point FFTs of C_A columns n1 each ------------
      constexpr int R = F::RA, T = F::TA, C = F::CA;
      const int col = tid % C;
      const int j = tid / C;
      const int c = (a.slab0 + slab) / a.Nss;
      const int sp = (a.slab0 + slab) % a.Nss;
      using W = typename SampleWord<FMT, NV>::type;
      const W* src0 = reinterpret_cast<const W*>(a.in) + (long long)c * a.chan_stride + (long long)sp * N + col +
                      (long long)N1 * j;
      W w[R];
      {
        const W* src = src0 + titem * K * C;
#pragma unroll
        for (int m = 0; m < R; ++m) w[m] = HintLoad<W>::ld(src + (long long)N1 * T * m, pol_first);
      }
#pragma unroll 1
      for (int t = 0; t < K; ++t) {
        const int n1 = (titem * K + t) * C + col;
        W wn[R];  // next tile's samples, requested before this tile's FFTs
        if (t + 1 < K) {
          const W* src = src0 + (titem * K + t + 1) * C;
#pragma unroll
          for (int m = 0; m < R; ++m) wn[m] = HintLoad<W>::ld(src + (long long)N1 * T * m, pol_first);
        }
        const int e0 = n1 * j;
        const float2 w0 = cmul(__ldg(a.twLo + (e0 & ((1 << a.h) - 1))), __ldg(a.twHi + (e0 >> a.h)));
        float2* dst = scr + n1;
        const float2* twm = a.twM + n1;
#pragma unroll
        for (int q = 0; q < NV; ++q) {
          float2 v[1][R];
#pragma unroll
          for (int m = 0; m < R; ++m) {
            float2 smp[NV];
            Unpack<FMT, NV>::run(w[m], smp);
            v[0][m] = q == 0 ? smp[0] : smp[NV - 1];
          }
          GroupFFT<N2, R, 1>::run(v, j, xch + (size_t)col * F::GSA, smem_padded_len(N2), twA, Sync{});
#pragma unroll
          for (int m = 0; m < R; ++m) {
            const int k2 = j + m * T;
            const float2 tw = m == 0 ? w0 : cmul(w0, __ldg(twm + (size_t)m * N1));
            st_f2_hint(dst + ((size_t)q * N2 + k2) * N1, cmul(v[0][m], tw), pol_last);
          }
        }
        if (t + 1 < K) {
#pragma unroll
          for (int m = 0; m < R; ++m) w[m] = wn[m];
        }
      }
      publish(doneA + slab, K);
    } else {
      wait_count(doneA + slab, tilesA, err, 2);
      // ---- K row tiles: N1-point FFTs of C_B rows k2, detection, store ----
      constexpr int R = F::RB, T = F::TB, C = F::CB;
      const int row = tid % C;
      const int j = tid / C;
      const int c = (a.slab0 + slab) / a.units_per_chan;
      const int d = (a.slab0 + slab) % a.units_per_chan;
      float* obase = a.out + ((size_t)d * NP * a.Nc + c) * N;
      const size_t plane = (size_t)a.Nc * N;
#pragma unroll 1
      for (int t = 0; t < K; ++t) {
        const int k2 = (titem * K + t) * C + row;
        const float2* src = scr + (size_t)k2 * N1 + j;
        // Polarisation 0, then 1; total power accumulates |X|^2 of each, the
        // cross-pol modes keep X0 while X1 is transformed.
        float2 x0[NV == 2 && POL != POL_TP ? R : 1];
        float tp[POL == POL_TP ? R : 1];
        float2 v[1][R];
#pragma unroll
        for (int q = 0; q < NV; ++q) {
#pragma unroll
          for (int m = 0; m < R; ++m) v[0][m] = ld_f2_hint(src + (size_t)q * N2 * N1 + m * T, pol_first);
          GroupFFT<N1, R, 1>::run(v, j, xch + (size_t)row * F::GSB, smem_padded_len(N1), twB, Sync{});
          if constexpr (POL == POL_TP) {
#pragma unroll
            for (int m = 0; m < R; ++m) {
              float t1[1] = {q == 0 ? 0.0f : tp[m]};
              const float2 xx[1] = {v[0][m]};
              detect_acc<POL_TP, 1>(t1, xx, im_sign);
              tp[m] = t1[0];
            }
          } else {
            if (q == 0) {
#pragma unroll
              for (int m = 0; m < R; ++m) x0[m] = v[0][m];
            }
          }
        }
        // Detection and store, MC bins at a time: in accumulate mode the
        // MC*NP old values are all requested before the first store.
        constexpr int MC = NP == 1 ? 8 : 4;
#pragma unroll
        for (int m0 = 0; m0 < R; m0 += MC) {
          float old[MC][NP];
          if (a.mode == ACC_ADD) {
#pragma unroll
            for (int mm = 0; mm < MC; ++mm) {
              const int pos = out_pos(k2 + N2 * (j + (m0 + mm) * T), N, a.inverse);
#pragma unroll
              for (int p = 0; p < NP; ++p) old[mm][p] = ld_f_hint(obase + p * plane + pos, pol_first);
            }
          }
#pragma unroll
          for (int mm = 0; mm < MC; ++mm) {
            const int m = m0 + mm;
            float acc[NP];
            if constexpr (POL == POL_TP) {
              acc[0] = tp[m];
            } else {
#pragma unroll
              for (int p = 0; p < NP; ++p) acc[p] = 0.0f;
              const float2 x[2] = {x0[m], v[0][m]};
              detect_acc<POL, 2>(acc, x, im_sign);
            }
            const int pos = out_pos(k2 + N2 * (j + m * T), N, a.inverse);
#pragma unroll
            for (int p = 0; p < NP; ++p) {
              const float val = a.mode == ACC_ADD ? __fmaf_rn(acc[p], a.scale, old[mm][p]) : acc[p] * a.scale;
              st_f_hint(obase + p * plane + pos, val, pol_first);
            }
          }
        }
      }
      publish(doneB + slab, K);
    }
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

template <int N1, int N2, int NV, int POL>
cudaError_t fused_t(const LargeLaunch& L, cudaStream_t s, int mode_op, int* ctas_out) {
  using F = FusedCfg<N1, N2, NV, POL>;
  auto k = k_large_fused<N1, N2, FMT_I8, NV, POL>;
  if (mode_op == 1) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F::SMEM);
  if (mode_op == 2) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFusedTPB, F::SMEM);
    if (e != cudaSuccess) return e;
    *ctas_out = std::max(1, per_sm) * sms;
    return cudaSuccess;
  }
  k<<<L.fused_ctas, kFusedTPB, F::SMEM, s>>>(L);
  return cudaGetLastError();
}

template <int N1, int N2>
cudaError_t fused_pol(const LargeLaunch& L, cudaStream_t s, int op, int* ctas) {
  if (L.nv == 1) return fused_t<N1, N2, 1, POL_TP>(L, s, op, ctas);
  switch (L.pol) {
    case POL_FULL: return fused_t<N1, N2, 2, POL_FULL>(L, s, op, ctas);
    case POL_STOKES: return fused_t<N1, N2, 2, POL_STOKES>(L, s, op, ctas);
    default: return fused_t<N1, N2, 2, POL_TP>(L, s, op, ctas);
  }
}

cudaError_t fused_dispatch(const LargeLaunch& L, cudaStream_t s, int op, int* ctas) {
  switch (L.logN) {
    case 16: return fused_pol<256, 256>(L, s, op, ctas);
    case 17: return fused_pol<256, 512>(L, s, op, ctas);
    case 18: return fused_pol<512, 512>(L, s, op, ctas);
    case 19: return fused_pol<512, 1024>(L, s, op, ctas);
    case 20: return fused_pol<1024, 1024>(L, s, op, ctas);
    case 21: return fused_pol<1024, 2048>(L, s, op, ctas);
    case 22: return fused_pol<2048, 2048>(L, s, op, ctas);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool large_fused_supported(const LargeLaunch& L) {
  return L.fmt == FMT_I8 && L.M == 1 && L.logN >= 16 && L.logN <= 22 && L.logN2 == (L.logN + 1) / 2;
}

int large_fused_ring() { return kRingSlots; }

int large_fused_row_radix(int pol) { return pol == POL_TP ? fused_rb<POL_TP>() : fused_rb<POL_FULL>(); }

int large_fused_col_radix() { return fused_ra(); }

int large_fused_ctl_ints(const LargeLaunch& L) { return 2 + 2 * L.Nc * L.Nss; }

cudaError_t large_fused_prepare(LargeLaunch& L) {
  cudaError_t e = fused_dispatch(L, nullptr, 1, nullptr);
  if (e != cudaSuccess) return e;
  return fused_dispatch(L, nullptr, 2, &L.fused_ctas);
}

cudaError_t large_fused_launch(const LargeLaunch& L, cudaStream_t s) {
  // reset the item counter and the per-slab counters; ctl[0] keeps errors
  cudaError_t e = cudaMemsetAsync(L.ctl + 1, 0, sizeof(int) * (size_t)(large_fused_ctl_ints(L) - 1), s);
  if (e != cudaSuccess) return e;
  return fused_dispatch(L, s, 0, nullptr);
}

}  // namespace rsg
