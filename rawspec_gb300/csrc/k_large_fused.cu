// k_large_fused.cu -- persistent four-step FFT spectrometer for long
// transforms whose integration unit is one spectrum per buffer (the case of
// the 2^20-point product of the production configuration).
//
// The two passes of the four-step FFT (see k_large.cu) become work items of
// one persistent kernel, taken in a fixed order through an atomic counter
// (shown for a lag of 2):
//
//   A(0) A(1) A(2) B(0) A(3) B(1) ... A(S-1) B(S-3) B(S-2) B(S-1)
//
// where A(s) are the column tiles of slab s (one channel-spectrum, both
// polarisations) and B(s) its row tiles.  A(s) writes the FP32 intermediate
// into slot s mod RING of a ring of RING slabs; B(s) waits until every A(s)
// tile is published, A(s) waits until every B(s-RING) tile has released the
// slot.  LAG and RING are chosen at plan time to cover the items in flight.
// An item only ever waits for items earlier in the order, which were taken
// by CTAs that are running, so the waits always end; they are bounded
// nonetheless and record an error instead of hanging if the bound is ever
// reached.
//
// Data movement.  Every tile's input reaches shared memory through the
// copy engine of the SM (TMA), double-buffered: the column tiles' 8-bit
// words as a 2-D tensor copy ([N2 rows] x [C_A words], rows N1 words apart),
// the row tiles' intermediate rows as 1-D bulk copies, one stage per
// polarisation.  A stage's buffer becomes the transform's exchange buffer
// once its values are in registers, and the next stage is requested as soon
// as the transform is done with it; the first two stages of the CTA's next
// work item (taken at that moment) are requested while the current one
// finishes, so the loads of one item overlap the arithmetic of the other.
// Completion is tracked by two mbarriers (expected-transaction counts).
// Intermediate rows are discarded from L2 once copied (they are dead), so
// rows still in L2 are never written back to HBM.
#include <cuda.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cstdlib>

#include "detect.cuh"
#include "fft_core.cuh"
#include "internal.h"

namespace rsg {

namespace {

constexpr int kFusedTPB = 256;
// Row tiles of slab s are queued after the column tiles of slab s + lag, and
// a slot of the intermediate ring is reused `ring` slabs later (ring > lag
// keeps every wait pointed at earlier items).  Both distances are chosen at
// plan time (large_fused_plan) to exceed the items in flight, so that a row
// tile rarely finds its column tiles still running and a column tile rarely
// finds its slot still in use.
// Tiles per work item (amortises the item overheads): 4 in total-power mode,
// 2 in the cross-pol modes (measured best on GB300 at 2^20).
#ifndef RSG_FUSED_K_TP
#define RSG_FUSED_K_TP 4
#endif
#ifndef RSG_FUSED_K_X
#define RSG_FUSED_K_X 2
#endif
template <int POL>
__host__ __device__ constexpr int fused_k() { return POL == POL_TP ? RSG_FUSED_K_TP : RSG_FUSED_K_X; }
static_assert(fused_k<POL_TP>() >= 2 && fused_k<POL_FULL>() >= 2, "an item must fill both stage buffers");
#ifndef RSG_FUSED_DISCARD
#define RSG_FUSED_DISCARD 1
#endif
constexpr long long kSpinLimit = 1ll << 24;         // polls of a counter (~2 s with back-off)
constexpr long long kMbarCycles = 4000000000ll;     // ~2 s of SM clocks for a stage copy

// Radix (values per thread per transform) of the column and row tiles.
#ifndef RSG_FUSED_RA
#define RSG_FUSED_RA 16
#endif
#ifndef RSG_FUSED_RB_TP
#define RSG_FUSED_RB_TP 16
#endif
#ifndef RSG_FUSED_RB_X
#define RSG_FUSED_RB_X 16
#endif
__host__ __device__ constexpr int fused_ra() { return RSG_FUSED_RA; }
template <int POL>
__host__ __device__ constexpr int fused_rb() { return POL == POL_TP ? RSG_FUSED_RB_TP : RSG_FUSED_RB_X; }

// Shared-memory distance between the exchange buffers of neighbouring
// interleaved sub-FFTs, chosen so that the C sub-FFTs served by one
// half-warp land on disjoint banks, and even (16-byte aligned rows for the
// bulk copies).
__host__ __device__ constexpr int group_stride(int N, int C) {
  int base = smem_padded_len(N);
  const int cp = C < 16 ? C : 16;
  const int want = (16 / cp) % 16;
  while (base % 16 != want) ++base;
  return base + (base & 1);
}

__host__ __device__ constexpr int round16(int x) { return (x + 15) & ~15; }

template <int N1, int N2, int POL>
struct FusedCfg {
  static constexpr int RA = fused_ra(), TA = N2 / RA, CA = kFusedTPB / TA;
  static constexpr int RB = fused_rb<POL>(), TB = N1 / RB, CB = kFusedTPB / TB;
  static constexpr int TWA = stockham_tw_size(N2, RA), TWB = stockham_tw_size(N1, RB);
  static constexpr int GSA = group_stride(N2, CA), GSB = group_stride(N1, CB);
  // column-tile words: boxes of BOXR rows x CW words (CW >= 4: 16-byte rows)
  static constexpr int CW = CA < 4 ? 4 : CA;
  static constexpr int BOXR = N2 < 256 ? N2 : 256;
  // row-tile outputs through tensor stores: total power (one plane) with rows
  // of at least 16 bytes; boxes of BOXO spectrum rows x C_B bins
  static constexpr bool TMA_OUT = POL == POL_TP && CB >= 4;
  static constexpr int BOXO = N1 / 2 < 256 ? N1 / 2 : 256;
  static constexpr int XCH = round16(CA * GSA > CB * GSB ? CA * GSA : CB * GSB);  // float2 per stage buffer
  static constexpr int TWS = round16((TA + RA) * CA);   // float2: column-tile twiddle slices per stage
  static constexpr int OUTS = TMA_OUT ? round16(CB * N1 / 2) : 0;  // float2: staged row-tile outputs
  static constexpr int OFF_TWB = round16(TWA), OFF_STG = OFF_TWB + round16(TWB);
  static constexpr int OFF_TWS = OFF_STG + 2 * XCH, OFF_OUT = OFF_TWS + 2 * TWS;
  static constexpr size_t SMEM = (size_t)(OFF_OUT + OUTS) * sizeof(float2) + 128;  // + alignment slack
  // Ring layout: the intermediate of a polarisation is stored in blocks of
  // BK consecutive k2, [k2 / BK][n1][k2 % BK].  With BK = C_B a row tile's
  // input is one contiguous block (one bulk copy) and a warp's column-tile
  // store covers whole 128-byte lines (its 32 / C_A values of j span the
  // block); where a warp spans fewer than C_B values of j, BK = 1 (rows).
  static constexpr int BK = (CB <= 32 / CA) ? CB : 1;
  // With BK = C_B the two polarisations are interleaved, [k2 / BK][n1][k2 %
  // BK] of 16 bytes (re pol 0, re pol 1, im pol 0, im pol 1: the packed pair
  // as the registers hold it): a column tile stores both values of a bin
  // with one 16-byte store, a row tile's input is one contiguous block of
  // both polarisations that lands in two halves of N1 / 2 values n1 (one per
  // stage buffer), and a row thread reads both values with one 16-byte load.
  static constexpr bool IL = BK == CB && (N1 / 2) % TB == 0;
  static constexpr unsigned BYTES_A = (unsigned)N2 * CW * 4;
  static constexpr unsigned BYTES_TW = (unsigned)(TA + RA) * CA * 8;
  static constexpr unsigned BYTES_B = (unsigned)CB * N1 * 8;
  static_assert(TA * CA == kFusedTPB && TB * CB == kFusedTPB, "sub-FFT threads must tile the CTA");
  static_assert((size_t)BYTES_A <= (size_t)XCH * sizeof(float2), "column words must fit a stage buffer");
  static_assert(N2 % BOXR == 0 && CA % 2 == 0, "tensor boxes must tile the column");
  static_assert(N1 % (2 * BOXO) == 0, "output boxes must not straddle the FFT shift");
};

// Offset of element (k2, n1) of polarisation q within a ring slot.
template <int N1, int N2, int BK>
__device__ __forceinline__ size_t ring_index(int q, int k2, int n1) {
  return ((size_t)q * N2 + (size_t)(k2 / BK) * BK) * N1 + (size_t)n1 * BK + (k2 % BK);
}

// Offset, in float4 (both polarisations of a value), of element (k2, n1) in
// the interleaved layout of a ring slot.
template <int N1, int BK>
__device__ __forceinline__ size_t ring_index_il(int k2, int n1) {
  return (size_t)(k2 / BK) * BK * N1 + (size_t)n1 * BK + (k2 % BK);
}

struct Sync {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

__device__ __forceinline__ int load_acquire(const int* p) {
  int v;
  asm volatile("ld.acquire.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// A bounded wait that runs out records its code in the error word and sets
// the CTA's abort flag: from then on the CTA issues no copy, skips every
// wait, finishes its current work item on whatever the buffers hold (all
// accesses stay in bounds), drains the copies already in flight and exits.
__device__ __forceinline__ void set_abort(int* err, int code, int* abort_flag) {
  atomicExch(err, code);
  *reinterpret_cast<volatile int*>(abort_flag) = 1;
}
__device__ __forceinline__ bool aborted(const int* abort_flag) {
  return *reinterpret_cast<const volatile int*>(abort_flag) != 0;
}

// Thread 0 polls until *cnt reaches target (bounded), then the CTA proceeds.
__device__ __forceinline__ void wait_count(const int* cnt, int target, int* err, int code, int* abort_flag) {
  if (threadIdx.x == 0 && !aborted(abort_flag)) {
    unsigned ns = 32;
    long long it = 0;
    while (load_acquire(cnt) < target) {
      if (++it > kSpinLimit) {
        set_abort(err, code, abort_flag);
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
__device__ __forceinline__ void st_f2_hint(float2* p, float2 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v2.f32 [%0], {%1, %2}, %3;" ::"l"(p), "f"(v.x), "f"(v.y), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_f4_hint(float4* p, float4 v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
               "f"(v.w), "l"(pol)
               : "memory");
}
__device__ __forceinline__ void st_f_hint(float* p, float v, unsigned long long pol) {
  asm volatile("st.global.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}
// *p += v, performed in L2 without returning a value (no wait on the thread).
__device__ __forceinline__ void red_add_f_hint(float* p, float v, unsigned long long pol) {
  asm volatile("red.global.add.L2::cache_hint.f32 [%0], %1, %2;" ::"l"(p), "f"(v), "l"(pol) : "memory");
}

// ---- mbarrier and bulk-copy primitives (PTX ISA: mbarrier, cp.async.bulk) ----
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(unsigned long long* mb, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(mb)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void mbar_expect_tx(unsigned long long* mb, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(mb)), "r"(bytes)
               : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* mb, unsigned parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_addr(mb)), "r"(parity)
      : "memory");
  return ok != 0;
}
// Waits for the phase of the given parity to complete (bounded by SM clock
// cycles; see set_abort).  Returns false if it ran out.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* mb, unsigned parity) {
  if (mbar_try_wait(mb, parity)) return true;
  const long long t0 = clock64();
  while (!mbar_try_wait(mb, parity)) {
    if (clock64() - t0 > kMbarCycles) return false;
  }
  return true;
}
__device__ __forceinline__ void mbar_wait(unsigned long long* mb, unsigned parity, int* err, int* abort_flag) {
  if (aborted(abort_flag)) return;
  if (!mbar_wait_bounded(mb, parity)) set_abort(err, 3, abort_flag);
}
// Orders this CTA's earlier generic-proxy accesses of shared memory before
// later asynchronous-proxy (copy engine) writes to it.
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, unsigned long long* mb,
                                            unsigned long long policy) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes.L2::cache_hint"
      " [%0], [%1, {%2, %3}], [%4], %5;" ::"r"(smem_addr(dst)),
      "l"(reinterpret_cast<unsigned long long>(map)), "r"(x), "r"(y), "r"(smem_addr(mb)), "l"(policy)
      : "memory");
}
__device__ __forceinline__ void bulk_load(void* dst, const void* src, unsigned bytes, unsigned long long* mb) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(smem_addr(mb))
               : "memory");
}
// Tensor stores from shared memory: plain (first buffer of an integration)
// or reduce-add into the accumulator (later buffers); one bulk group per tile.
__device__ __forceinline__ void tma_store_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.async.bulk.tensor.2d.global.shared::cta.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<unsigned long long>(map)),
               "r"(x), "r"(y), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void tma_reduce_add_2d(const CUtensorMap* map, int x, int y, const void* src) {
  asm volatile("cp.reduce.async.bulk.tensor.2d.global.shared::cta.add.bulk_group [%0, {%1, %2}], [%3];" ::"l"(
                   reinterpret_cast<unsigned long long>(map)),
               "r"(x), "r"(y), "r"(smem_addr(src))
               : "memory");
}
__device__ __forceinline__ void bulk_commit() { asm volatile("cp.async.bulk.commit_group;" ::: "memory"); }
// The bulk groups committed so far have finished reading shared memory.
__device__ __forceinline__ void bulk_wait_read() { asm volatile("cp.async.bulk.wait_group.read 0;" ::: "memory"); }
// The bulk groups committed so far are complete.
__device__ __forceinline__ void bulk_wait_all() { asm volatile("cp.async.bulk.wait_group 0;" ::: "memory"); }
// The 128-byte L2 line at p holds dead data: drop it without writing it back.
__device__ __forceinline__ void discard_l2(const void* p) {
  asm volatile("discard.global.L2 [%0], 128;" ::"l"(p) : "memory");
}

// A work item: K consecutive column tiles (A) or row tiles (B) of one slab.
// Segment k of the order holds A(k) (k < S) followed by B(k - lag) (k >= lag).
struct Item {
  bool isA;
  int slab, titem;
};
__device__ __forceinline__ Item decode_item(long long item, int S, int lag, int itemsA, int itemsB) {
  Item it;
  const int p1 = S < lag ? S : lag;       // A-only segments
  const int mid = S > lag ? S - lag : 0;  // A+B segments
  const long long n1 = (long long)p1 * itemsA;
  const long long n2 = (long long)mid * (itemsA + itemsB);
  if (item < n1) {
    it.isA = true;
    it.slab = (int)(item / itemsA);
    it.titem = (int)(item % itemsA);
  } else if (item < n1 + n2) {
    const long long i2 = item - n1;
    const int k = lag + (int)(i2 / (itemsA + itemsB));
    const int r = (int)(i2 % (itemsA + itemsB));
    it.isA = r < itemsA;
    it.slab = it.isA ? k : k - lag;
    it.titem = it.isA ? r : r - itemsA;
  } else {  // B-only tail
    const long long i3 = item - n1 - n2;
    it.isA = false;
    it.slab = mid + (int)(i3 / itemsB);
    it.titem = (int)(i3 % itemsB);
  }
  return it;
}

}  // namespace

// TOUT: row-tile outputs through tensor stores (total power, forward
// transforms, F::TMA_OUT); otherwise per-thread stores (and loads of the
// accumulator in accumulate mode).
template <int N1, int N2, int POL, bool TOUT>
__global__ void __launch_bounds__(kFusedTPB, 2)
k_large_fused(const __grid_constant__ LargeLaunch a) {
  using F = FusedCfg<N1, N2, POL>;
  static_assert(!TOUT || F::TMA_OUT, "tensor-store outputs need one plane and 16-byte rows");
  constexpr int N = N1 * N2;
  constexpr int NP = PolOut<POL>::NP;
  constexpr int K = fused_k<POL>();
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* twA = reinterpret_cast<float2*>((reinterpret_cast<uintptr_t>(smem_raw) + 127) & ~uintptr_t(127));
  float2* twB = twA + F::OFF_TWB;
  float2* stg = twA + F::OFF_STG;  // two stage buffers of F::XCH float2
  float2* tws = twA + F::OFF_TWS;  // two twiddle-slice buffers of F::TWS float2
  float* outs = reinterpret_cast<float*>(twA + F::OFF_OUT);  // [N1 shifted rows][C_B bins]
  __shared__ __align__(8) unsigned long long mbar[2];
  __shared__ long long s_next;
  __shared__ int s_pre;
  __shared__ int s_abort;
  __shared__ unsigned s_issued[2];  // stages thread 0 has requested into each buffer

  const int tid = threadIdx.x;
  const int S = a.S;
  constexpr int tilesA = N1 / F::CA, tilesB = N2 / F::CB;
  static_assert(tilesA % K == 0 && tilesB % K == 0, "items must cover whole tiles");
  constexpr int itemsA = tilesA / K, itemsB = tilesB / K;
  const long long total = (long long)S * (itemsA + itemsB);
  int* err = a.ctl;  // sticky error word (never reset by a launch)
  int* exited = a.ctl + 1;  // CTAs of this launch that have finished
  int* next = a.ctl + 2;
  int* doneA = a.ctl + 3;
  int* doneB = a.ctl + 3 + S;
  const float im_sign = a.conj ? -1.0f : 1.0f;
  const unsigned long long pol_first = policy_evict_first();
  const unsigned long long pol_last = policy_evict_last();

  if (tid == 0) {
    mbar_init(&mbar[0], 1);
    mbar_init(&mbar[1], 1);
    mbar_init_fence();
    s_next = (long long)atomicAdd(reinterpret_cast<unsigned int*>(next), 1u);
    s_pre = 0;
    s_abort = 0;
    s_issued[0] = s_issued[1] = 0;
  }
  for (int i = tid; i < F::TWA; i += kFusedTPB) twA[i] = a.twN2[i];
  for (int i = tid; i < F::TWB; i += kFusedTPB) twB[i] = a.twN1[i];
  __syncthreads();

  // Stage copies (issued by thread 0).  Column stage t of an item: the C_A
  // columns of tile titem*K + t, all N2 rows, as 8-bit words, plus the
  // tile's twiddle slices; row stage s: polarisation s%2 of the C_B rows of
  // tile titem*K + s/2, from the ring.
  auto issue_stage = [&](const Item& it, int s, int buf) {
    if (aborted(&s_abort)) return;
    ++s_issued[buf];
    float2* dst = stg + (size_t)buf * F::XCH;
    unsigned long long* mb = &mbar[buf];
    if (it.isA) {
      const int tile = it.titem * K + s;
      const long long gs = (long long)a.slab0 + it.slab;
      const long long row0 = ((gs / a.Nss) * a.chan_stride + (gs % a.Nss) * (long long)N) / N1;
      const int x0 = (tile * F::CA) & ~3;  // 16-byte aligned start column
      mbar_expect_tx(mb, F::BYTES_A + F::BYTES_TW);
      uint32_t* words = reinterpret_cast<uint32_t*>(dst);
#pragma unroll 1
      for (int i = 0; i < N2 / F::BOXR; ++i)
        tma_load_2d(words + (size_t)i * F::BOXR * F::CW, &a.tmap_in, x0, (int)(row0 + (long long)i * F::BOXR), mb,
                    pol_first);
      float2* tw = tws + (size_t)buf * F::TWS;
      tma_load_2d(tw, &a.tmap_twj, tile * F::CA, 0, mb, pol_last);
      tma_load_2d(tw + F::TA * F::CA, &a.tmap_twm, tile * F::CA, 0, mb, pol_last);
    } else {
      const int tile = it.titem * K + (s >> 1);
      const int q = s & 1;  // interleaved: half q of the tile's block; else polarisation q
      const float2* slotp = a.scratch + (size_t)(it.slab % a.ring) * 2 * N;
      const float2* src = F::IL ? slotp + ((size_t)2 * tile + q) * F::CB * N1
                                : slotp + ((size_t)q * N2 + (size_t)tile * F::CB) * N1;
      mbar_expect_tx(mb, F::BYTES_B);
      if constexpr (F::BK == F::CB) {
        bulk_load(dst, src, F::BYTES_B, mb);  // one block [n1][C_B rows]
      } else {
#pragma unroll 1
        for (int r = 0; r < F::CB; ++r) bulk_load(dst + (size_t)r * F::GSB, src + (size_t)r * N1, N1 * 8, mb);
      }
    }
  };

  unsigned ph = 0;  // bit b: parity of the next completion of stage buffer b
  bool pre_ok = false;  // thread 0: the next item's first stages are in flight
  for (;;) {
    __syncthreads();  // the previous item's s_next / s_pre are written
    const long long item = s_next;
    const int pre = s_pre;
    const int abort_now = s_abort;
    __syncthreads();
    if (item >= total || abort_now) break;
    const Item it = decode_item(item, S, a.lag, itemsA, itemsB);
    long long nxt = total;
    if (tid == 0) pre_ok = false;
    const int nstages = it.isA ? K : 2 * K;
    // Requests stage s + 2 into the buffer stage s has released: the item's
    // own, else the next item's first stages (B only once its column tiles
    // are all published).  The next item is taken here, when the first of
    // them is due, so that each CTA holds little more than one item at a
    // time.  Called by every thread after a CTA barrier that follows the last
    // use of the buffer.
    auto refill = [&](int s) {
      if (tid != 0) return;
      const int buf = s & 1;
      if (s + 2 < nstages) {
        fence_proxy_async();
        issue_stage(it, s + 2, buf);
        return;
      }
      if (s + 2 == nstages) {
        nxt = (long long)atomicAdd(reinterpret_cast<unsigned int*>(next), 1u);
        s_next = nxt;
        if (nxt < total) {
          const Item nit = decode_item(nxt, S, a.lag, itemsA, itemsB);
          pre_ok = nit.isA || load_acquire(doneA + nit.slab) >= tilesA;
        }
      }
      if (pre_ok) {
        fence_proxy_async();
        issue_stage(decode_item(nxt, S, a.lag, itemsA, itemsB), s + 2 - nstages, buf);
      }
    };

    const int slot = it.slab % a.ring;
    float2* scr = a.scratch + (size_t)slot * 2 * N;

    if (it.isA) {
      if (tid == 0 && !pre) {
        fence_proxy_async();
        issue_stage(it, 0, 0);
        issue_stage(it, 1, 1);
      }
      if (it.slab >= a.ring) wait_count(doneB + (it.slab - a.ring), tilesB, err, 1, &s_abort);
      // ---- K column tiles: N2-point FFTs of C_A columns n1 each ------------
      constexpr int R = F::RA, T = F::TA, C = F::CA;
      const int col = tid % C;
      const int j = tid / C;
#pragma unroll 1
      for (int t = 0; t < K; ++t) {
        const int buf = t & 1;
        float2* sb = stg + (size_t)buf * F::XCH;
        const float2* tw = tws + (size_t)buf * F::TWS;  // [T][C] then [R][C]
        mbar_wait(&mbar[buf], (ph >> buf) & 1u, err, &s_abort);
        ph ^= 1u << buf;
        const int tile = it.titem * K + t;
        const int n1 = tile * C + col;
        const uint32_t* words = reinterpret_cast<const uint32_t*>(sb) + ((tile * C) & 3) + col;
        // both polarisations in lockstep on the packed instructions
        cpair v[R];
#pragma unroll
        for (int m = 0; m < R; ++m) {
          float2 smp[2];
          Unpack<FMT_I8, 2>::run(words[(j + T * m) * F::CW], smp);
          v[m] = pack2(smp[0], smp[1]);
        }
        __syncthreads();  // the buffer becomes the exchange buffer; tile t-1 is done
        if (t > 0) refill(t - 1);
        const float2 w0 = tw[j * C + col];  // W_N^(n1 j)
        float2* dst = scr;
        GroupFFT<N2, R, 2>::template run_packed<true>(v, j, sb + (size_t)col * F::GSA, 0, twA, Sync{});
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const int k2 = j + m * T;
          // W_N^(n1 k2) = W_N^(n1 j) W_N^(n1 m T)
          const float2 twk = m == 0 ? w0 : cmul(w0, tw[(T + m) * C + col]);
          const cpair x = pmul(v[m], twk);
          if constexpr (F::IL) {
            st_f4_hint(reinterpret_cast<float4*>(dst) + ring_index_il<N1, F::BK>(k2, n1),
                       make_float4(x.re.x, x.re.y, x.im.x, x.im.y), pol_last);
          } else {
            st_f2_hint(dst + ring_index<N1, N2, F::BK>(0, k2, n1), lane0(x), pol_last);
            st_f2_hint(dst + ring_index<N1, N2, F::BK>(1, k2, n1), lane1(x), pol_last);
          }
        }
      }
      publish(doneA + it.slab, K);
      refill(K - 1);
    } else {
      if (!pre) {
        wait_count(doneA + it.slab, tilesA, err, 2, &s_abort);
        if (tid == 0) {
          fence_proxy_async();
          issue_stage(it, 0, 0);
          issue_stage(it, 1, 1);
        }
      }
      // ---- K row tiles: N1-point FFTs of C_B rows k2, detection, store ----
      constexpr int R = F::RB, T = F::TB, C = F::CB;
      const int row = tid % C;
      const int j = tid / C;
      const int c = (a.slab0 + it.slab) / a.units_per_chan;
      const int d = (a.slab0 + it.slab) % a.units_per_chan;
      float* obase = a.out + ((size_t)d * NP * a.Nc + c) * N;
      const size_t plane = (size_t)a.Nc * N;
      // where element n1 of this thread's row sits in a landed stage
      auto row_slot = [&](int n1) -> size_t {
        if constexpr (F::BK == C) return (size_t)n1 * C + row;
        else return (size_t)row * F::GSB + n1;
      };
#pragma unroll 1
      for (int t = 0; t < K; ++t) {
        const int tile = it.titem * K + t;
        const int k2 = tile * C + row;
        float2 x0[POL != POL_TP ? R : 1];
        float tp[POL == POL_TP ? R : 1];
        float2 v[1][R];
        // Both polarisations (stage 2t in buffer 0, stage 2t+1 in buffer 1)
        // into registers as packed pairs, transformed in lockstep with the
        // exchanges in buffer 1; buffer 0 is refilled before the transform,
        // buffer 1 after it.
        {
          float2* sb0 = stg;
          float2* sb1 = stg + F::XCH;
          cpair vp[R];
          mbar_wait(&mbar[0], ph & 1u, err, &s_abort);
          ph ^= 1u;
          if constexpr (F::IL) {
            // values n1 < N1/2 in buffer 0, the others in buffer 1
            constexpr int MH = N1 / 2 / T;
            const float4* h0 = reinterpret_cast<const float4*>(sb0) + (size_t)j * C + row;
            const float4* h1 = reinterpret_cast<const float4*>(sb1) + (size_t)j * C + row;
#pragma unroll
            for (int m = 0; m < MH; ++m) {
              const float4 f = h0[(size_t)m * T * C];
              vp[m] = cpair{make_float2(f.x, f.y), make_float2(f.z, f.w)};
            }
            mbar_wait(&mbar[1], (ph >> 1) & 1u, err, &s_abort);
            ph ^= 2u;
#pragma unroll
            for (int m = MH; m < R; ++m) {
              const float4 f = h1[(size_t)(m - MH) * T * C];
              vp[m] = cpair{make_float2(f.x, f.y), make_float2(f.z, f.w)};
            }
          } else {
#pragma unroll
            for (int m = 0; m < R; ++m) v[0][m] = sb0[row_slot(j + m * T)];
            mbar_wait(&mbar[1], (ph >> 1) & 1u, err, &s_abort);
            ph ^= 2u;
#pragma unroll
            for (int m = 0; m < R; ++m) vp[m] = pack2(v[0][m], sb1[row_slot(j + m * T)]);
          }
#if RSG_FUSED_DISCARD
          if constexpr (F::IL) {
            const char* blk = reinterpret_cast<const char*>(scr + (size_t)2 * tile * C * N1);
            constexpr int kLines = 2 * F::BYTES_B / 128;
#pragma unroll 1
            for (int l = tid; l < kLines; l += kFusedTPB) discard_l2(blk + (size_t)l * 128);
          } else {
            const char* rows0 = reinterpret_cast<const char*>(scr + (size_t)tile * C * N1);
            const char* rows1 = reinterpret_cast<const char*>(scr + ((size_t)N2 + (size_t)tile * C) * N1);
            constexpr int kLines = F::BYTES_B / 128;
#pragma unroll 1
            for (int l = tid; l < kLines; l += kFusedTPB) {
              discard_l2(rows0 + (size_t)l * 128);
              discard_l2(rows1 + (size_t)l * 128);
            }
          }
#endif
          // the previous tile's output copy must have read the staging area
          if (TOUT && tid == 0) bulk_wait_read();
          __syncthreads();  // both stage buffers are read
          refill(2 * t);
          GroupFFT<N1, R, 2>::template run_packed<true>(vp, j, sb1 + (size_t)row * F::GSB, 0, twB, Sync{});
          refill(2 * t + 1);
          if constexpr (POL == POL_TP) {
#pragma unroll
            for (int m = 0; m < R; ++m) {
              const float2 pw = f2fma(vp[m].im, vp[m].im, f2mul(vp[m].re, vp[m].re));
              tp[m] = pw.x + pw.y;
            }
          } else {
            // cross products: x0 = (|X0|^2, |X1|^2) from the packed pair,
            // v[0] = (Re, Im)(X0 X1*)
#pragma unroll
            for (int m = 0; m < R; ++m) {
              const float2 a0 = lane0(vp[m]), a1 = lane1(vp[m]);
              x0[m] = f2fma(vp[m].im, vp[m].im, f2mul(vp[m].re, vp[m].re));
              v[0][m] = make_float2(__fmaf_rn(a0.y, a1.y, a0.x * a1.x), __fmaf_rn(-a0.x, a1.y, a0.y * a1.x));
            }
          }
        }
        if constexpr (TOUT) {
          // Shifted bin k2 + N2*((k1 + N1/2) mod N1): staged as
          // [row (k1 + N1/2) mod N1][k2 - tile*C], then written (first
          // buffer) or added (later buffers) by tensor copies.
#pragma unroll
          for (int m = 0; m < R; ++m) {
            const int k1s = (j + m * T + N1 / 2) & (N1 - 1);
            outs[k1s * C + row] = tp[m] * a.scale;
          }
          fence_proxy_async();
          __syncthreads();
          if (tid == 0) {
            const int y0 = (int)(((long long)d * NP * a.Nc + c) * N1);
#pragma unroll 1
            for (int i = 0; i < N1 / F::BOXO; ++i) {
              if (a.mode == ACC_ADD)
                tma_reduce_add_2d(&a.tmap_out, tile * C, y0 + i * F::BOXO, outs + i * F::BOXO * C);
              else
                tma_store_2d(&a.tmap_out, tile * C, y0 + i * F::BOXO, outs + i * F::BOXO * C);
            }
            bulk_commit();
          }
          continue;
        }
        // Detection and store: written (first buffer of an integration) or
        // added in L2 (later buffers), one value per bin and plane.
#pragma unroll
        for (int m = 0; m < R; ++m) {
          float acc[NP];
          if constexpr (POL == POL_TP) {
            acc[0] = tp[m];
          } else {
            acc[0] = POL == POL_FULL ? x0[m].x : x0[m].x + x0[m].y;
            acc[1] = POL == POL_FULL ? x0[m].y : x0[m].x - x0[m].y;
            acc[2] = v[0][m].x;
            acc[3] = im_sign * v[0][m].y;
          }
          const int pos = out_pos(k2 + N2 * (j + m * T), N, a.inverse);
#pragma unroll
          for (int p = 0; p < NP; ++p) {
            if (a.mode == ACC_ADD)
              red_add_f_hint(obase + p * plane + pos, acc[p] * a.scale, pol_first);
            else
              st_f_hint(obase + p * plane + pos, acc[p] * a.scale, pol_first);
          }
        }
      }
      publish(doneB + it.slab, K);
    }
    if (tid == 0) s_pre = pre_ok ? 1 : 0;
  }
  // Copies still in flight complete before the CTA retires: after a normal
  // run every requested stage has been waited for; after an abort, the last
  // stage requested into each buffer is waited for (bounded; the phases of an
  // mbarrier complete in order, so the earlier ones are then complete too).
  if (tid == 0) {
    for (int b = 0; b < 2; ++b)
      if (s_issued[b] > 0 && !mbar_wait_bounded(&mbar[b], (s_issued[b] - 1) & 1u)) atomicExch(err, 4);
  }
  if (TOUT && tid == 0) bulk_wait_all();
  // The last CTA to finish zeroes the counters for the next launch (every
  // other CTA has stopped reading them); the error word stays.
  __shared__ int s_last;
  __syncthreads();
  if (tid == 0) {
    __threadfence();
    s_last = atomicAdd(exited, 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    for (int i = tid; i < 1 + 2 * S; i += kFusedTPB) next[i] = 0;
    if (tid == 0) *exited = 0;
    __threadfence();
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

template <int N1, int N2, int POL>
cudaError_t fused_t(const LargeLaunch& L, cudaStream_t s, int mode_op, int* ctas_out) {
  using F = FusedCfg<N1, N2, POL>;
  auto k = (F::TMA_OUT && !L.inverse) ? k_large_fused<N1, N2, POL, F::TMA_OUT> : k_large_fused<N1, N2, POL, false>;
  if (mode_op == 1) {
    cudaError_t e = cudaFuncSetAttribute(k_large_fused<N1, N2, POL, false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, (int)F::SMEM);
    if (e != cudaSuccess || !F::TMA_OUT) return e;
    return cudaFuncSetAttribute(k_large_fused<N1, N2, POL, F::TMA_OUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                (int)F::SMEM);
  }
  if (mode_op == 2) {
    int dev = 0, sms = 0, per_sm = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, kFusedTPB, F::SMEM);
    if (e != cudaSuccess) return e;
    *ctas_out = std::max(1, per_sm) * sms;
    return cudaSuccess;
  }
  if (mode_op == 3) {  // tensor-map geometry
    ctas_out[0] = F::CW;
    ctas_out[1] = F::BOXR;
    ctas_out[2] = F::CA;
    ctas_out[3] = F::TA;
    ctas_out[4] = F::RA;
    ctas_out[5] = F::CB;
    ctas_out[6] = F::BOXO;
    ctas_out[7] = F::TMA_OUT ? 1 : 0;
    ctas_out[8] = fused_k<POL>();
    return cudaSuccess;
  }
  k<<<L.fused_ctas, kFusedTPB, F::SMEM, s>>>(L);
  return cudaGetLastError();
}

template <int N1, int N2>
cudaError_t fused_pol(const LargeLaunch& L, cudaStream_t s, int op, int* ctas) {
  switch (L.pol) {
    case POL_FULL: return fused_t<N1, N2, POL_FULL>(L, s, op, ctas);
    case POL_STOKES: return fused_t<N1, N2, POL_STOKES>(L, s, op, ctas);
    default: return fused_t<N1, N2, POL_TP>(L, s, op, ctas);
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

PFN_cuTensorMapEncodeTiled_v12000 tensor_map_encoder() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
  }
  return fn;
}

}  // namespace

bool large_fused_supported(const LargeLaunch& L) {
  if (L.fmt != FMT_I8 || L.nv != 2 || L.M != 1 || L.logN < 16 || L.logN > 22) return false;
  if (L.logN2 != (L.logN + 1) / 2) return false;
  const long long n1 = 1ll << L.logN1;
  // the column tiles' tensor copies view each channel as rows of N1 words
  return L.chan_stride % n1 == 0 && (reinterpret_cast<uintptr_t>(L.in) & 15) == 0;
}

cudaError_t large_fused_plan(LargeLaunch& L) {
  cudaError_t e = fused_dispatch(L, nullptr, 1, nullptr);  // shared-memory limit first: occupancy depends on it
  if (e != cudaSuccess) return e;
  e = fused_dispatch(L, nullptr, 2, &L.fused_ctas);
  if (e != cudaSuccess) return e;
  int geo[9] = {0};
  e = fused_dispatch(L, nullptr, 3, geo);
  if (e != cudaSuccess) return e;
  // Items in flight: about 1.5 per CTA (the one it works on, and the next
  // one, taken shortly before the current one ends).  A segment of the order
  // holds one slab's column and row items; lag and ring - lag both span at
  // least the items in flight.
  const int CA = geo[2], CB = geo[5];
  const long long seg = (long long)((1 << L.logN1) / CA + (1 << L.logN2) / CB) / geo[8];
  const int d = (int)((3ll * L.fused_ctas / 2 + seg - 1) / seg);
#ifdef RSG_FUSED_LAG
  L.lag = RSG_FUSED_LAG;
#else
  L.lag = std::max(2, d);
#endif
#ifdef RSG_FUSED_RING
  L.ring = RSG_FUSED_RING;
#else
  L.ring = std::max(L.lag + 2, L.lag + d);
#endif
  L.lag_pipe = L.lag;
  if (const char* v = getenv("RAWSPEC_GB300_FUSED_LAG_PIPE")) L.lag_pipe = std::max(1, std::min(L.ring - 1, atoi(v)));
  return L.ring > L.lag ? cudaSuccess : cudaErrorInvalidValue;
}

int large_fused_row_radix(int pol) { return pol == POL_TP ? fused_rb<POL_TP>() : fused_rb<POL_FULL>(); }

int large_fused_col_radix() { return fused_ra(); }

int large_fused_ctl_ints(const LargeLaunch& L) { return 3 + 2 * L.Nc * L.Nss; }

namespace {

// 2-D tensor map: rows of `width` elements of `esize` bytes, `pitch` bytes apart.
cudaError_t encode_2d(CUtensorMap* map, const void* base, CUtensorMapDataType type, int esize,
                      unsigned long long width, unsigned long long rows, unsigned long long pitch, int box_w,
                      int box_h) {
  PFN_cuTensorMapEncodeTiled_v12000 enc = tensor_map_encoder();
  if (!enc) return cudaErrorNotSupported;
  (void)esize;
  cuuint64_t dims[2] = {(cuuint64_t)width, (cuuint64_t)rows};
  cuuint64_t strides[1] = {(cuuint64_t)pitch};
  cuuint32_t box[2] = {(cuuint32_t)box_w, (cuuint32_t)box_h};
  cuuint32_t estr[2] = {1, 1};
  CUresult r = enc(map, type, 2, const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                   CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  return r == CUDA_SUCCESS ? cudaSuccess : cudaErrorInvalidValue;
}

}  // namespace

int large_fused_twj_entries(const LargeLaunch& L) {
  return (1 << L.logN1) * ((1 << L.logN2) / fused_ra());
}

cudaError_t large_fused_prepare(LargeLaunch& L) {
  cudaError_t e = fused_dispatch(L, nullptr, 1, nullptr);
  if (e != cudaSuccess) return e;
  e = fused_dispatch(L, nullptr, 2, &L.fused_ctas);
  if (e != cudaSuccess) return e;
  int geo[9] = {0};
  e = fused_dispatch(L, nullptr, 3, geo);
  if (e != cudaSuccess) return e;
  const int CW = geo[0], BOXR = geo[1], CA = geo[2], TA = geo[3], RA = geo[4], CB = geo[5], BOXO = geo[6];
  const unsigned long long n1 = 1ull << L.logN1, n2 = 1ull << L.logN2;
  // the input buffer as rows of N1 32-bit words (one word: a sample of both
  // polarisations)
  e = encode_2d(&L.tmap_in, L.in, CU_TENSOR_MAP_DATA_TYPE_UINT32, 4, n1, (unsigned long long)L.Nc * L.chan_stride / n1,
                n1 * 4, CW, BOXR);
  if (e != cudaSuccess) return e;
  // twiddle tables [T_A][N1] (W_N^(n1 j)) and [R_A][N1] (W_N^(n1 m T_A)), 8-byte entries
  e = encode_2d(&L.tmap_twj, L.twJ, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, n1, (unsigned long long)TA, n1 * 8, CA, TA);
  if (e != cudaSuccess) return e;
  e = encode_2d(&L.tmap_twm, L.twM, CU_TENSOR_MAP_DATA_TYPE_FLOAT64, 8, n1, (unsigned long long)RA, n1 * 8, CA, RA);
  if (e != cudaSuccess) return e;
  // the dump buffer [units][|P|][Nc][N] as rows of N2 floats (total power)
  if (geo[7]) {
    const unsigned long long rows = (unsigned long long)L.units_per_chan * L.Nc * n1;
    e = encode_2d(&L.tmap_out, L.out, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, n2, rows, n2 * 4, CB, BOXO);
    if (e != cudaSuccess) return e;
  }
  return cudaSuccess;
}

cudaError_t large_fused_launch(const LargeLaunch& L, cudaStream_t s) {
  // the counters were zeroed at initialisation and are zeroed again by the
  // last CTA of every launch
  return fused_dispatch(L, s, 0, nullptr);
}

}  // namespace rsg
