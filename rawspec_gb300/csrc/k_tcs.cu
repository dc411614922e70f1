// k_tcs.cu -- spectrometer product kernel for short transforms (N = 8, 16,
// 32) whose DFT runs on the tensor cores in one stage (tcgen05, FP16
// operands, FP32 accumulation in tensor memory), for 8-bit input of two
// polarisations.
//
// Like k_small and k_tc it replaces the reference's per-(product, batch,
// pol) cufftExecC2C calls with their texture load callback and store
// callbacks (rawspec_gpu.cu:1555-1569, :133-267), the sub-integration
// `accumulate` kernel (:297-318) and the FFT-shifting copies (:1647-1697).
//
// The whole N-point DFT is one GEMM: a 128-row data operand (row 2 s + p =
// polarisation p of spectrum s of the tile, columns the (re, im) codes of
// its N samples, exact in FP16) times the real 2N x 2N form of the DFT
// matrix, split as hi + lo in FP16 (about 22 significant bits together).
// The MMAs against both halves accumulate into the same tensor-memory
// columns, so the thread owning lane 2 s + p reads X_p[k] of spectrum s for
// every k.  Detection needs the other polarisation only for the cross
// products, and it sits in the neighbouring lane (one shuffle).
//
// A CTA works through its tiles of 64 spectra (each of one integration
// unit) as one stream.  Warp 4 is the producer: one thread copies the input
// tiles into a ring of shared-memory stages (bulk copies, several tiles
// ahead) and issues each tile's MMAs once the consumers have written its
// data operand.  Warps 0-3 are the consumers, one thread per tensor-memory
// lane: they convert tile g into one of two data operands while the MMAs of
// tile g-1 run, then detect tile g-1, handing over through mbarriers only.
// Each consumer accumulates its lane's powers over the unit's tiles in
// registers; at the end of the unit the lanes and warps are summed in a
// fixed order and the FFT-shifted spectrum is stored (or a partial sum per
// chunk of the unit, finished by k_finalize).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cuda_fp16.h>
#include <type_traits>

#include "detect.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace rsg {

template <int N>
struct TcsCfg {
  static constexpr int K = 2 * N;            // contraction: (re, im) of the N samples of one polarisation
  static constexpr int ND = 2 * N;           // MMA N: the N outputs x (re, im)
  static constexpr int NB = 4 * N;           // rows of the DFT operand: [hi | lo] x ND
  static constexpr int LBO = 128;            // core matrices along K
  static constexpr int SBO = (K / 8) * LBO;  // 8-row groups
  static constexpr int A_BYTES = 16 * SBO;   // one 128 x K data operand
  static constexpr int B_BYTES = (NB / 8) * SBO;
  static constexpr int B_LO = (ND / 8) * SBO;  // the lo half
  static constexpr int CONSUMERS = 128;      // warps 0-3: one thread per tensor-memory lane
  static constexpr int THREADS = 160;        // + warp 4: the input copies and the MMAs
  static constexpr int SPT = 64;             // spectra per tile (x 2 polarisations = 128 rows)
  static constexpr int TILE_BYTES = SPT * N * 4;  // a tile's input words
  static constexpr int STAGES = N == 8 ? 6 : N == 16 ? 4 : 3;  // input tiles in flight
  static constexpr int ACC_COLS = ND < 32 ? 32 : ND;  // tensor-memory columns per accumulator
  static constexpr int TMEM_COLS = 2 * ACC_COLS;      // two tiles in flight
  static constexpr int RED_FLOATS = 4 * 4 * N;        // [warp][plane][bin]
  // data operands x 2 | DFT operand | input stages | reduction areas x 2 |
  // mbarriers: input landed x STAGES, operand ready x 2, MMAs done x 2 |
  // tensor-memory slot, abort flag, commit counters x 2, copy counters x STAGES
  static constexpr int OFF_IN = 2 * A_BYTES + B_BYTES;
  static constexpr int OFF_RED = OFF_IN + STAGES * TILE_BYTES;
  static constexpr int OFF_BAR = OFF_RED + 2 * RED_FLOATS * (int)sizeof(float);
  static constexpr int SMEM = OFF_BAR + 8 * (STAGES + 4) + 4 * (4 + STAGES);
  static_assert(N % 8 == 0 && N <= 32, "lengths 8, 16, 32");
};

namespace {

constexpr long long kTcsWaitCycles = 2000000000ll;  // ~1 s of SM clocks for an MMA batch or a tile copy

// Sums v over the 32 lanes of the warp, leaving lane l with the sum of
// element l >> (5 - log2 CNT) (CNT <= 32): each halving step keeps the half
// selected by one lane bit and adds the partner's copy of it (CNT - 1
// shuffles), the remaining lane bits are summed whole.
template <int CNT>
__device__ __forceinline__ float warp_transpose_sum(float (&v)[CNT], int lane) {
  constexpr int LOG = CNT == 1 ? 0 : CNT == 2 ? 1 : CNT == 4 ? 2 : CNT == 8 ? 3 : CNT == 16 ? 4 : 5;
  static_assert((1 << LOG) == CNT && LOG <= 5, "a power of two up to 32");
#pragma unroll
  for (int st = 0; st < LOG; ++st) {
    const int half = CNT >> (st + 1), off = 16 >> st;
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float mine = upper ? v[half + i] : v[i];
      const float other = upper ? v[i] : v[half + i];
      v[i] = mine + __shfl_xor_sync(0xffffffffu, other, off);
    }
  }
  float s = v[0];
#pragma unroll
  for (int off = 16 >> LOG; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
  return s;
}

// The same over the lanes of one parity (lane bit 0 kept apart), CNT >= 16:
// four halving steps leave lane l with elements ((l >> 1) & 15) * CNT/16 + r,
// r < CNT/16, summed over the 16 lanes of its parity.
template <int CNT>
__device__ __forceinline__ void warp_transpose_sum_parity(float (&v)[CNT], int lane) {
  static_assert(CNT >= 16, "four halving steps");
#pragma unroll
  for (int st = 0; st < 4; ++st) {
    const int half = CNT >> (st + 1), off = 16 >> st;
    const bool upper = (lane & off) != 0;
#pragma unroll
    for (int i = 0; i < half; ++i) {
      const float mine = upper ? v[half + i] : v[i];
      const float other = upper ? v[i] : v[half + i];
      v[i] = mine + __shfl_xor_sync(0xffffffffu, other, off);
    }
  }
}

}  // namespace

template <int N, int POL>
__global__ void __launch_bounds__(TcsCfg<N>::THREADS) k_tcs(const __grid_constant__ TcLaunch a) {
  using C = TcsCfg<N>;
  constexpr int NP = PolOut<POL>::NP, SPT = C::SPT, ST = C::STAGES;
  constexpr uint32_t IDESC = tc::idesc_f16_f32(128, C::ND);
  // total power: (sum x^2, sum y^2) per bin on the packed instructions;
  // cross products: two planes per lane (polarisation-0 lanes planes 0 and
  // 2, polarisation-1 lanes planes 1 and 3)
  constexpr int NACC = POL == POL_TP ? N : 2 * N;
  using Acc = typename std::conditional<POL == POL_TP, float2, float>::type;
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned char* sA = sm;                   // two data operands
  unsigned char* sB = sm + 2 * C::A_BYTES;  // DFT operand [hi | lo]
  unsigned char* sIn = sm + C::OFF_IN;      // input stages
  float* red = reinterpret_cast<float*>(sm + C::OFF_RED);  // two [warp][plane][bin] areas
  uint64_t* full = reinterpret_cast<uint64_t*>(sm + C::OFF_BAR);  // input stage landed (copy)
  uint64_t* opready = full + ST;   // data operand written, accumulator read (4 consumer warps)
  uint64_t* mmadone = opready + 2; // the tile's MMAs complete (commit)
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mmadone + 2);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tslot + 1);
  uint32_t* ncommit = tslot + 2;   // commits issued to mmadone[0], [1] (producer)
  uint32_t* nissue = ncommit + 2;  // copies issued into each stage (producer)

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int items = a.unit_count * a.chunks;
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.tab);
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = tid; i < C::B_BYTES / 16; i += C::THREADS) dst[i] = __ldg(src + i);
  }
  if (tid == 0) {
    for (int s = 0; s < ST; ++s) {
      tc::mbar_init(full + s, 1);
      nissue[s] = 0;
    }
    for (int b = 0; b < 2; ++b) {
      tc::mbar_init(opready + b, 4);
      tc::mbar_init(mmadone + b, 1);
      ncommit[b] = 0;
    }
    *abort_flag = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, C::TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;

  // A bounded wait that runs out sets the abort flag; from then on every
  // wait returns at once, no copy or MMA is issued, and both roles run their
  // loops to the end on whatever the buffers hold (all accesses stay in
  // bounds); the teardown waits for what is still in flight.
  auto wait = [&](uint64_t* b, unsigned parity) {
    if (*abort_flag) return;
    if (!tc::mbar_wait_bounded(b, parity, kTcsWaitCycles)) *abort_flag = 1;
  };
  auto tiles_of = [&](int item) {
    const int s_begin = (item % a.chunks) * a.spc;
    return (min(a.M, s_begin + a.spc) - s_begin) / SPT;
  };

  if (warp == 4) {
    // ---- producer: the input copies, ST tiles ahead, and the MMAs ----
    if (lane == 0) {
      const uint32_t aA = tc::smem_u32(sA), bF = tc::smem_u32(sB), bFlo = bF + C::B_LO;
      int i_item = blockIdx.x, i_t = 0, i_nt = 0;
      const uint32_t* i_src = nullptr;  // the next tile to copy
      unsigned issued = 0;
      auto start_item = [&]() {
        if (i_item >= items) return;
        const int unit = a.unit0 + i_item / a.chunks, chunk = i_item % a.chunks;
        const int c = unit / a.units_per_chan, d = unit % a.units_per_chan;
        i_nt = tiles_of(i_item);
        i_src = reinterpret_cast<const uint32_t*>(a.in) + (long long)c * a.chan_stride +
                ((long long)d * a.M + (long long)chunk * a.spc) * N;
      };
      auto issue_in = [&]() {
        if (i_item >= items) return;
        if (!*abort_flag) {
          const int s = issued % ST;
          tc::mbar_arrive_expect_tx(full + s, C::TILE_BYTES);
          tc::bulk_load(sIn + s * C::TILE_BYTES, i_src, C::TILE_BYTES, full + s);
          ++nissue[s];
        }
        ++issued;
        i_src += SPT * N;
        if (++i_t >= i_nt) {
          i_item += gridDim.x;
          i_t = 0;
          start_item();
        }
      };
      start_item();
      for (int s = 0; s < ST; ++s) issue_in();
      int m_item = blockIdx.x, m_t = 0, m_nt = m_item < items ? tiles_of(m_item) : 0;
      for (unsigned g = 0; m_item < items; ++g) {
        const int b = g & 1;
        // operand b holds tile g and accumulator b has been read (tile g-2)
        wait(opready + b, (g >> 1) & 1u);
        tc::fence_after_sync();
        if (!*abort_flag) {
          const uint32_t d = tmem + b * C::ACC_COLS, aa = aA + b * C::A_BYTES;
#pragma unroll
          for (int ks = 0; ks < C::K / 16; ++ks)
            tc::mma_f16(d, tc::smem_desc(aa + ks * 2 * C::LBO, C::LBO, C::SBO),
                        tc::smem_desc(bF + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, ks > 0 ? 1u : 0u);
#pragma unroll
          for (int ks = 0; ks < C::K / 16; ++ks)
            tc::mma_f16(d, tc::smem_desc(aa + ks * 2 * C::LBO, C::LBO, C::SBO),
                        tc::smem_desc(bFlo + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, 1u);
          tc::mma_commit(mmadone + b);
          ++ncommit[b];
        }
        issue_in();  // tile g's input stage has been read: tile g + ST goes there
        if (++m_t >= m_nt) {
          m_item += gridDim.x;
          m_t = 0;
          m_nt = m_item < items ? tiles_of(m_item) : 0;
        }
      }
    }
    __syncwarp();
  } else {
    // ---- consumers: row tid = polarisation pol of spectrum sp of the tile ----
    const uint32_t lane_off = (uint32_t)(warp * 32) << 16;  // this warp's lanes
    const int sp = tid >> 1, pol = tid & 1;
    const uint32_t sel = pol ? 0x4342u : 0x4140u;
    const float im_sign = a.conj ? -1.0f : 1.0f;

    // input stage of tile g -> data operand b: samples 4c .. 4c+3 of the
    // row as (re, im) FP16 pairs fill core matrix c of the row
    auto convert = [&](unsigned g, int b) {
      const int s = g % ST;
      wait(full + s, (g / ST) & 1u);
      const uint4* w = reinterpret_cast<const uint4*>(sIn + s * C::TILE_BYTES) + sp * (N / 4);
      unsigned char* row = sA + b * C::A_BYTES + (tid >> 3) * C::SBO + (tid & 7) * 16;
#pragma unroll
      for (int c = 0; c < N / 4; ++c) {
        const uint4 q = w[c];
        const uint32_t x[4] = {q.x, q.y, q.z, q.w};
        uint32_t h[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) h[i] = tc::codes_to_h2(__vmaxs4(x[i], 0x81818181u) ^ 0x80808080u, sel);
        *reinterpret_cast<uint4*>(row + c * C::LBO) = make_uint4(h[0], h[1], h[2], h[3]);
      }
    };
    // waits for tile g's MMAs (accumulator g % 2) and adds its detected values
    auto detect = [&](unsigned g, Acc (&acc)[NACC]) {
      const int b = g & 1;
      wait(mmadone + b, (g >> 1) & 1u);
      tc::fence_after_sync();
      const uint32_t d = tmem + b * C::ACC_COLS + lane_off;
#pragma unroll
      for (int ch = 0; ch < C::ND / 16; ++ch) {
        float h[16];
        tc::tmem_ld16(d + 16 * ch, h);
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const int k = 8 * ch + i;
          const float2 X = make_float2(h[2 * i], h[2 * i + 1]);
          if constexpr (POL == POL_TP) {
            acc[k] = __ffma2_rn(X, X, acc[k]);
          } else {
            const float2 Y =
                make_float2(__shfl_xor_sync(0xffffffffu, X.x, 1), __shfl_xor_sync(0xffffffffu, X.y, 1));
            const float2 x0 = pol ? Y : X, x1 = pol ? X : Y;
            const float p0 = __fmaf_rn(x0.x, x0.x, x0.y * x0.y);
            const float p1 = __fmaf_rn(x1.x, x1.x, x1.y * x1.y);
            if (!pol) {
              acc[k] += POL == POL_FULL ? p0 : p0 + p1;
              acc[N + k] += __fmaf_rn(x0.x, x1.x, x0.y * x1.y);
            } else {
              acc[k] += POL == POL_FULL ? p1 : p0 - p1;
              acc[N + k] = __fmaf_rn(im_sign, __fmaf_rn(x0.y, x1.x, -(x0.x * x1.y)), acc[N + k]);
            }
          }
        }
      }
    };
    // the unit's (chunk's) spectrum from the lanes' sums: lanes, then warps,
    // in a fixed order, through reduction area f % 2 (the consumers' named
    // barrier of the next use of the other area orders these reads before
    // this area's next writes); acc is cleared for the next unit
    auto finish = [&](int item, Acc (&acc)[NACC], int f) {
      float* r = red + (f & 1) * C::RED_FLOATS;
      const int unit = a.unit0 + item / a.chunks, chunk = item % a.chunks;
      const int c = unit / a.units_per_chan, d = unit % a.units_per_chan;
      if constexpr (POL == POL_TP) {
        float v[N];
#pragma unroll
        for (int k = 0; k < N; ++k) v[k] = acc[k].x + acc[k].y;
        const float s = warp_transpose_sum<N>(v, lane);
        constexpr int SH = N == 8 ? 2 : N == 16 ? 1 : 0;  // 5 - log2 N
        if ((lane & ((1 << SH) - 1)) == 0) r[warp * N + (lane >> SH)] = s;
      } else {
        warp_transpose_sum_parity<2 * N>(acc, lane);
        constexpr int RL = 2 * N / 16;
#pragma unroll
        for (int q = 0; q < RL; ++q) {
          const int j = ((lane >> 1) & 15) * RL + q;
          r[(warp * 4 + pol + (j < N ? 0 : 2)) * N + (j % N)] = acc[q];
        }
      }
#pragma unroll
      for (int i = 0; i < NACC; ++i) acc[i] = Acc{};
      asm volatile("bar.sync 1, %0;" ::"n"(C::CONSUMERS) : "memory");
      for (int o = tid; o < NP * N; o += C::CONSUMERS) {
        const int pl = o / N, k = o - pl * N;
        float s = 0.0f;
#pragma unroll
        for (int wq = 0; wq < 4; ++wq) s += r[(wq * NP + pl) * N + k];
        if (a.chunks > 1) {
          a.partial[(((size_t)unit * a.chunks + chunk) * NP + pl) * N + k] = s;
        } else {
          float* dst = a.out + (((size_t)d * NP + pl) * a.Nc + c) * N + out_pos(k, N, a.inverse);
          if (a.mode == ACC_ADD) *dst = __fmaf_rn(s, a.scale, *dst); else *dst = s * a.scale;
        }
      }
    };

    // The CTA's tiles as one stream, two in flight: tile g is converted while
    // the MMAs of tile g-1 run, then tile g-1 is detected (across the units'
    // boundaries too, so that a unit's end exposes no MMA latency).
    Acc acc[NACC];
#pragma unroll
    for (int i = 0; i < NACC; ++i) acc[i] = Acc{};
    int c_item = blockIdx.x, c_t = 0, c_nt = c_item < items ? tiles_of(c_item) : 0;
    int p_item = -1, nfin = 0;
    bool p_last = false;  // the previous tile ends its item
    unsigned g = 0;
    for (; c_item < items; ++g) {
      // operand g % 2 was read by the MMAs of tile g-2, accumulator g % 2 by
      // this thread's loads when tile g-2 was detected (both done by now)
      convert(g, g & 1);
      tc::fence_proxy_async_smem();
      tc::fence_before_sync();
      __syncwarp();
      if (lane == 0) tc::mbar_arrive(opready + (g & 1));
      if (p_item >= 0) {
        detect(g - 1, acc);
        if (p_last) finish(p_item, acc, nfin++);
      }
      p_item = c_item;
      p_last = c_t + 1 == c_nt;
      if (++c_t >= c_nt) {
        c_item += gridDim.x;
        c_t = 0;
        c_nt = c_item < items ? tiles_of(c_item) : 0;
      }
    }
    if (p_item >= 0) {
      detect(g - 1, acc);
      finish(p_item, acc, nfin++);
    }
  }

  // No MMA is still running and no copy is still landing when the tensor
  // memory and the CTA's shared memory are released: after a normal run the
  // consumers have waited for every commit and every copy; after a time-out
  // the producer waits (bounded) for the last commit of each MMA barrier and
  // the last copy of each stage (an mbarrier's phases complete in order).
  __syncthreads();
  if (tid == 4 * 32 && *abort_flag) {
    for (int b = 0; b < 2; ++b)
      if (ncommit[b] > 0) tc::mbar_wait_bounded(mmadone + b, (ncommit[b] - 1) & 1u, kTcsWaitCycles);
    for (int s = 0; s < ST; ++s)
      if (nissue[s] > 0) tc::mbar_wait_bounded(full + s, (nissue[s] - 1) & 1u, kTcsWaitCycles);
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
  if (tid == 0 && *abort_flag) atomicExch(a.err, 1);
}

// The DFT operand in the byte layout of the kernel's shared memory: rows
// [hi | lo] x (k, re/im), columns (n, re/im); FP64 sincospi, hi = FP16(w),
// lo = FP16(w - hi).
template <int N>
__global__ void k_tcs_tables(unsigned char* tab) {
  using C = TcsCfg<N>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= C::NB * C::K) return;
  const int j = i / C::K, kk = i % C::K;
  const int h = j / C::ND, k = (j % C::ND) >> 1, cc = j & 1, n = kk >> 1, dd = kk & 1;
  double sn, cs;
  sincospi(2.0 * ((n * k) % N) / N, &sn, &cs);
  // W = cs - i sn;  (xr + i xi) W = (xr cs + xi sn) + i (xi cs - xr sn)
  const double v = cc == 0 ? (dd == 0 ? cs : sn) : (dd == 0 ? -sn : cs);
  const __half hv = __double2half(v);
  const __half out = h == 0 ? hv : __double2half(v - (double)__half2float(hv));
  *reinterpret_cast<__half*>(tab + (j >> 3) * C::SBO + (kk >> 3) * C::LBO + (j & 7) * 16 + (kk & 7) * 2) = out;
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

// Resident CTAs per SM: registers, shared memory, and the tensor-memory
// columns of the SM (the dynamic shared memory is padded so that no more
// CTAs than that fit).
template <int N, int POL>
cudaError_t tcs_plan_t(int* occ, size_t* smem) {
  using C = TcsCfg<N>;
  auto k = k_tcs<N, POL>;
  cudaFuncAttributes fa;
  int dev = 0, regs_sm = 0, smem_sm = 0, smem_rsv = 0;
  cudaError_t e;
  if ((e = cudaFuncGetAttributes(&fa, k)) != cudaSuccess || (e = cudaGetDevice(&dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess ||
      (e = cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
    return e;
  const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * C::THREADS;
  const int o = std::max(1, std::min({regs_sm / std::max(regs_cta, 1), 512 / C::TMEM_COLS,
                                      smem_sm / (C::SMEM + smem_rsv + (int)fa.sharedSizeBytes)}));
  const int per_cta = smem_sm / o - smem_rsv - (int)fa.sharedSizeBytes;
  if (per_cta < C::SMEM) return cudaErrorInvalidValue;
  *occ = o;
  *smem = (size_t)per_cta;
  if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, per_cta)) != cudaSuccess) return e;
  return cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
}

template <int N, int POL>
cudaError_t tcs_launch_t(const TcLaunch& L, cudaStream_t s) {
  const int items = L.unit_count * L.chunks;
  const int grid = std::min(items, std::max(L.slots, 1));
  if (grid < 1) return cudaSuccess;
  k_tcs<N, POL><<<grid, TcsCfg<N>::THREADS, L.smem, s>>>(L);
  return cudaGetLastError();
}

template <int N>
cudaError_t tcs_pol(const TcLaunch& L, cudaStream_t s, int op, int* occ, size_t* smem) {
  switch (L.pol) {
    case POL_TP: return op ? tcs_plan_t<N, POL_TP>(occ, smem) : tcs_launch_t<N, POL_TP>(L, s);
    case POL_FULL: return op ? tcs_plan_t<N, POL_FULL>(occ, smem) : tcs_launch_t<N, POL_FULL>(L, s);
    case POL_STOKES: return op ? tcs_plan_t<N, POL_STOKES>(occ, smem) : tcs_launch_t<N, POL_STOKES>(L, s);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t tcs_dispatch(const TcLaunch& L, cudaStream_t s, int op, int* occ = nullptr, size_t* smem = nullptr) {
  switch (L.logN) {
    case 3: return tcs_pol<8>(L, s, op, occ, smem);
    case 4: return tcs_pol<16>(L, s, op, occ, smem);
    case 5: return tcs_pol<32>(L, s, op, occ, smem);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

bool tcs_supported(int logN, int fmt, int nv, int pol, int M) {
  if (fmt != FMT_I8 || nv != 2 || logN < 3 || logN > 5) return false;
  if (pol != POL_TP && pol != POL_FULL && pol != POL_STOKES) return false;
  return M % TcsCfg<8>::SPT == 0;
}

size_t tcs_table_bytes(int logN) {
  switch (logN) {
    case 3: return TcsCfg<8>::B_BYTES;
    case 4: return TcsCfg<16>::B_BYTES;
    case 5: return TcsCfg<32>::B_BYTES;
    default: return 0;
  }
}

cudaError_t tcs_table_fill(void* dst, int logN, cudaStream_t s) {
  const size_t bytes = tcs_table_bytes(logN);
  if (!bytes) return cudaErrorInvalidValue;
  unsigned char* t = static_cast<unsigned char*>(dst);
  switch (logN) {
    case 3: k_tcs_tables<8><<<(TcsCfg<8>::NB * TcsCfg<8>::K + 255) / 256, 256, 0, s>>>(t); break;
    case 4: k_tcs_tables<16><<<(TcsCfg<16>::NB * TcsCfg<16>::K + 255) / 256, 256, 0, s>>>(t); break;
    default: k_tcs_tables<32><<<(TcsCfg<32>::NB * TcsCfg<32>::K + 255) / 256, 256, 0, s>>>(t); break;
  }
  return cudaGetLastError();
}

cudaError_t tcs_plan(const TcLaunch& L, int* occ, size_t* smem) { return tcs_dispatch(L, nullptr, 1, occ, smem); }

cudaError_t tcs_launch(const TcLaunch& L, cudaStream_t s) { return tcs_dispatch(L, s, 0); }

}  // namespace rsg
