// k_tc.cu -- spectrometer product kernel whose DFT runs on the tensor cores
// (tcgen05, FP16 operands, FP32 accumulation in tensor memory), for 8-bit
// input of two polarisations and N = S * S with S = 16, 32, 64.
//
// It replaces, like k_small, the reference's per-(product, batch, pol)
// cufftExecC2C calls with their texture load callback and read-modify-write
// store callbacks (rawspec_gpu.cu:1555-1569, :133-267), the sub-integration
// `accumulate` kernel (:297-318) and the FFT-shifting copies (:1647-1697).
//
// Four-step DFT with n = S n1 + n2, k = k1 + S k2:
//   stage 1  Y[k1][n2] = sum_n1 x[S n1 + n2] W_S^(n1 k1)
//   twiddle  T[k1][n2] = Y[k1][n2] W_N^(n2 k1)
//   stage 2  X[k1 + S k2] = sum_n2 T[k1][n2] W_S^(n2 k2)
// Each stage is one GEMM of a 128-row data operand (rows = sequences x S,
// columns = the (re, im) pairs of the S points) with the real 2S x 2S form of
// the S-point DFT matrix.  The DFT matrix is split as hi + lo in FP16 (about
// 22 significant bits together) and both halves are stacked along the MMA's
// N dimension, so one MMA yields both partial products side by side in the
// thread's own tensor-memory lane.  Stage-1 data are the integer codes,
// exact in FP16; the twiddled intermediate T is split into FP16 hi + lo and
// both halves enter stage 2.  The result carries about 22 bits per term,
// accumulated in FP32.
//
// A CTA (4 warps) works through tiles of 128 / S sequences (spectrum,
// polarisation): integer codes -> FP16 operand in shared memory -> stage-1
// MMAs -> twiddle and hi/lo split by the thread owning each tensor-memory
// lane -> stage-2 MMAs -> detection and accumulation of the unit's spectra in
// registers -> fixed-order reduction over the tile's sequences and an
// FFT-shifted store (or per-chunk partial sums, finished by k_finalize).
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cuda_fp16.h>

#include "detect.cuh"
#include "internal.h"
#include "tc_ptx.cuh"

namespace rsg {

template <int S>
struct TcCfg {
  static constexpr int N = S * S;
  static constexpr int K = 2 * S;             // contraction length: (re, im) of S points
  static constexpr int ND = 4 * S;            // MMA N: [hi | lo] x S outputs x (re, im)
  static constexpr int NSEQ = 128 / S;        // sequences (spectrum, polarisation) per tile
  static constexpr int SPT = NSEQ / 2;        // spectra per tile
  static constexpr int LBO = 144;             // core matrices along K: 128 bytes + 16 of padding
  static constexpr int SBO = (K / 8) * LBO;   // 8-row groups
  static constexpr int A_BYTES = 16 * SBO;    // one 128 x K data operand
  static constexpr int B_BYTES = (ND / 8) * SBO;
  static constexpr int TW_BYTES = N * 8;      // W_N^(n2 k1) as [k1][n2] float2
  static constexpr int TAB_BYTES = B_BYTES + TW_BYTES;
  // stage-1 operand | T hi | T lo | DFT operand | twiddles | 2 mbarriers,
  // tensor-memory slot, 2 commit counters
  static constexpr int SMEM = 3 * A_BYTES + TAB_BYTES + 32;
  static constexpr int TMEM_COLS = 2 * ND;    // stage-1 and stage-2 accumulators
  static constexpr int THREADS = 256;         // two warps per tensor-memory lane quarter
  static constexpr int MINB = S == 16 ? 3 : 512 / TMEM_COLS;
  static constexpr int WPT = S / 4;           // input words per thread per tile
  static_assert(SPT * S == 64, "64 (spectrum, n2) pairs per tile, four threads each");
  static_assert(4 * SPT * (int)sizeof(float) * N <= 3 * A_BYTES, "reduction fits the operand area");
};

namespace {

constexpr long long kTcWaitCycles = 2000000000ll;  // ~1 s of SM clocks for an MMA batch


}  // namespace

// Two tiles are in flight per CTA: the stage-1 MMAs of tile t+1 run while
// tile t is detected, and the stage-2 MMAs of tile t+1 while the codes of
// tile t+2 are converted.  Each accumulator (stage 1, stage 2) has its own
// tensor-memory columns and its own mbarrier; every shared-memory operand is
// rewritten only after the MMAs reading it have completed.  Warps w and w + 4
// read the same tensor-memory lanes and split the accumulator columns
// between them (8-column chunks q with q % 2 = w / 4).
template <int S, int POL>
__global__ void __launch_bounds__(TcCfg<S>::THREADS, TcCfg<S>::MINB) k_tc(const __grid_constant__ TcLaunch a) {
  using C = TcCfg<S>;
  constexpr int N = C::N, NSEQ = C::NSEQ, SPT = C::SPT, NP = PolOut<POL>::NP;
  constexpr int T = C::THREADS, NQ = S / 16;  // 8-column chunks per thread
  constexpr int NACC = POL == POL_TP ? S / 2 : S;
  constexpr uint32_t IDESC = tc::idesc_f16_f32(128, C::ND);      // against [F hi | F lo]
  constexpr uint32_t IDESC_HI = tc::idesc_f16_f32(128, C::ND / 2);  // against F hi alone
  static_assert(POL == POL_TP || S <= 32, "cross-pol modes keep 2 S accumulators per thread");
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned char* sA1 = sm;                   // stage-1 operand (integer codes)
  unsigned char* sAhi = sm + C::A_BYTES;     // T hi
  unsigned char* sAlo = sm + 2 * C::A_BYTES; // T lo
  unsigned char* sB = sm + 3 * C::A_BYTES;   // DFT operand [hi | lo], then the twiddles
  const float2* sTw = reinterpret_cast<const float2*>(sB + C::B_BYTES);
  uint64_t* mb1 = reinterpret_cast<uint64_t*>(sB + C::TAB_BYTES);
  uint64_t* mb2 = mb1 + 1;
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mb1 + 2);
  uint32_t* ncommit = tslot + 1;  // commits issued to mb1 and mb2 (thread 0)
  float* red = reinterpret_cast<float*>(sm);  // reduction area over the operands

  const int tid = threadIdx.x, warp = tid >> 5;
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.tab);
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = tid; i < C::TAB_BYTES / 16; i += T) dst[i] = __ldg(src + i);
  }
  if (tid == 0) {
    tc::mbar_init(mb1, 1);
    tc::mbar_init(mb2, 1);
    ncommit[0] = ncommit[1] = 0;
  }
  if (warp == 0) {
    tc::tmem_alloc(tslot, C::TMEM_COLS);
    tc::tmem_relinquish();
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  const uint32_t tmem = *tslot;
  const uint32_t d1 = tmem, d2 = tmem + C::ND;                       // accumulator columns
  const uint32_t lane_off = (uint32_t)((warp & 3) * 32) << 16;       // this warp's lanes
  const int half = warp >> 2;                                        // its column chunks
  const uint32_t aA1 = tc::smem_u32(sA1), aHi = tc::smem_u32(sAhi), aLo = tc::smem_u32(sAlo);
  const uint32_t bF = tc::smem_u32(sB);
  unsigned ph1 = 0, ph2 = 0;
  int bad = 0;  // one of this thread's waits timed out

  // input words: thread -> (spectrum of the tile, n2), a quarter of the n1 range
  const int pair = tid & 63, lsp = pair / S, ln2 = pair % S, n1_0 = (tid >> 6) * (S / 4);
  // tensor-memory lane of this thread: sequence seq, index r (n2 after stage
  // 1, k1 after stage 2)
  const int lane_row = tid & 127, seq = lane_row / S, r = lane_row % S;
  const float im_sign = a.conj ? -1.0f : 1.0f;

  uint32_t w[C::WPT];
  auto load = [&](const uint32_t* p) {
#pragma unroll
    for (int j = 0; j < C::WPT; ++j) w[j] = __ldg(p + j * S);
  };
  // stage-1 operand: rows (2 lsp + pol) S + n2, columns (n1, re/im)
  auto convert = [&]() {
#pragma unroll
    for (int g4 = 0; g4 < C::WPT / 4; ++g4) {
      uint32_t h0[4], h1[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t x = __vmaxs4(w[4 * g4 + i], 0x81818181u) ^ 0x80808080u;
        h0[i] = tc::codes_to_h2(x, 0x4140);
        h1[i] = tc::codes_to_h2(x, 0x4342);
      }
      const int kc = n1_0 / 4 + g4;
      const int m0 = (2 * lsp) * S + ln2, m1 = m0 + S;
      *reinterpret_cast<uint4*>(sA1 + (m0 >> 3) * C::SBO + kc * C::LBO + (m0 & 7) * 16) =
          make_uint4(h0[0], h0[1], h0[2], h0[3]);
      *reinterpret_cast<uint4*>(sA1 + (m1 >> 3) * C::SBO + kc * C::LBO + (m1 & 7) * 16) =
          make_uint4(h1[0], h1[1], h1[2], h1[3]);
    }
  };
  // operands written and earlier tensor-memory loads complete -> MMAs
  auto sync_for_mma = [&]() -> bool {
    tc::fence_proxy_async_smem();
    tc::fence_before_sync();
    const int stop = __syncthreads_or(bad);
    if (!stop && tid == 0) tc::fence_after_sync();
    return stop != 0;
  };
  auto issue_s1 = [&]() {
#pragma unroll
    for (int ks = 0; ks < C::K / 16; ++ks)
      tc::mma_f16(d1, tc::smem_desc(aA1 + ks * 2 * C::LBO, C::LBO, C::SBO),
                  tc::smem_desc(bF + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, ks > 0 ? 1u : 0u);
    tc::mma_commit(mb1);
    ++ncommit[0];
  };
  // T hi x [F hi | F lo] + T lo x F hi (the lo x lo term is below 2^-22)
  auto issue_s2 = [&]() {
#pragma unroll
    for (int ks = 0; ks < C::K / 16; ++ks)
      tc::mma_f16(d2, tc::smem_desc(aHi + ks * 2 * C::LBO, C::LBO, C::SBO),
                  tc::smem_desc(bF + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, ks > 0 ? 1u : 0u);
#pragma unroll
    for (int ks = 0; ks < C::K / 16; ++ks)
      tc::mma_f16(d2, tc::smem_desc(aLo + ks * 2 * C::LBO, C::LBO, C::SBO),
                  tc::smem_desc(bF + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC_HI, 1u);
    tc::mma_commit(mb2);
    ++ncommit[1];
  };
  auto wait = [&](uint64_t* mb, unsigned& ph) {
    if (!tc::mbar_wait_bounded(mb, ph, kTcWaitCycles)) bad = 1;
    ph ^= 1;
    tc::fence_after_sync();
  };
  // twiddle and hi/lo split: row seq S + k1, columns (n2 = r, re/im)
  auto epi1 = [&]() {
#pragma unroll
    for (int qq = 0; qq < NQ; ++qq) {
      const int q = 2 * qq + half;
      // the chunk's twiddles are read while its accumulator columns load
      float2 twv[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) twv[i] = sTw[(8 * q + i) * S + r];
      float h[16], l[16];
      tc::tmem_ld16x2(d1 + lane_off + 16 * q, d1 + lane_off + 2 * S + 16 * q, h, l);
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const int k1 = 8 * q + i;
        // (re, im) pairs on the packed instructions: y = hi + lo products,
        // y w, and the residual below the FP16 part
        const float2 y = __fadd2_rn(make_float2(h[2 * i], h[2 * i + 1]), make_float2(l[2 * i], l[2 * i + 1]));
        const float2 w = twv[i];
        const float2 tv = __ffma2_rn(make_float2(-y.y, y.y), make_float2(w.y, w.x),
                                     __fmul2_rn(make_float2(y.x, y.x), w));
        const __half2 hi = __floats2half2_rn(tv.x, tv.y);
        const float2 hf = __half22float2(hi);
        const float2 res = __ffma2_rn(hf, make_float2(-1.0f, -1.0f), tv);
        const __half2 lo = __floats2half2_rn(res.x, res.y);
        const int mr = seq * S + k1;
        const int off = (mr >> 3) * C::SBO + (r >> 2) * C::LBO + (mr & 7) * 16 + (r & 3) * 4;
        *reinterpret_cast<__half2*>(sAhi + off) = hi;
        *reinterpret_cast<__half2*>(sAlo + off) = lo;
      }
    }
  };
  // detection: lane seq S + k1 holds X[k1 + S k2] for all k2
  constexpr int NACC2 = POL == POL_TP ? S / 2 : 1;  // total power: packed (x^2, y^2) sums
  auto epi2 = [&](float (&acc)[NACC], float2 (&acc2)[NACC2]) {
#pragma unroll
    for (int qq = 0; qq < NQ; ++qq) {
      const int q = 2 * qq + half;
      float h[16], l[16];
      tc::tmem_ld16x2(d2 + lane_off + 16 * q, d2 + lane_off + 2 * S + 16 * q, h, l);
      float2 X[8];
#pragma unroll
      for (int i = 0; i < 8; ++i) X[i] = __fadd2_rn(make_float2(h[2 * i], h[2 * i + 1]), make_float2(l[2 * i], l[2 * i + 1]));
      if constexpr (POL == POL_TP) {
        // (sum x^2, sum y^2) per bin on the packed instructions
#pragma unroll
        for (int i = 0; i < 8; ++i) acc2[8 * qq + i] = __ffma2_rn(X[i], X[i], acc2[8 * qq + i]);
      } else {
        // the other polarisation of the same spectrum and k1 is lane tid ^ S
        float2 Y[8];
        if constexpr (S == 16) {
#pragma unroll
          for (int i = 0; i < 8; ++i) {
            Y[i].x = __shfl_xor_sync(0xffffffffu, X[i].x, 16);
            Y[i].y = __shfl_xor_sync(0xffffffffu, X[i].y, 16);
          }
        } else {
          // exchange through the T areas: their stage-2 MMAs have completed,
          // and they are rewritten only after the barrier that ends this phase
          float2* xb = reinterpret_cast<float2*>(sAhi) + (2 * half + (qq & 1)) * 128 * 8;
#pragma unroll
          for (int i = 0; i < 8; ++i) xb[i * 128 + lane_row] = X[i];
          __syncthreads();
#pragma unroll
          for (int i = 0; i < 8; ++i) Y[i] = xb[i * 128 + (lane_row ^ S)];
        }
        const bool p1 = (seq & 1) != 0;
#pragma unroll
        for (int i = 0; i < 8; ++i) {
          const float2 x0 = p1 ? Y[i] : X[i], x1 = p1 ? X[i] : Y[i];
          const float pw0 = __fmaf_rn(x0.x, x0.x, x0.y * x0.y);
          const float pw1 = __fmaf_rn(x1.x, x1.x, x1.y * x1.y);
          const int j = 8 * qq + i;
          if (!p1) {
            acc[j] += POL == POL_FULL ? pw0 : pw0 + pw1;
            acc[S / 2 + j] += __fmaf_rn(x0.x, x1.x, x0.y * x1.y);
          } else {
            acc[j] += POL == POL_FULL ? pw1 : pw0 - pw1;
            acc[S / 2 + j] = __fmaf_rn(im_sign, __fmaf_rn(x0.y, x1.x, -(x0.x * x1.y)), acc[S / 2 + j]);
          }
        }
      }
    }
    if constexpr (POL != POL_TP && S > 16) __syncthreads();
  };

  const int items = a.unit_count * a.chunks;
  bool stop = false;
  for (int item = blockIdx.x; item < items && !stop; item += gridDim.x) {
    const int unit = a.unit0 + item / a.chunks, chunk = item % a.chunks;
    const int c = unit / a.units_per_chan, d = unit % a.units_per_chan;
    const int s_begin = chunk * a.spc;
    const int s_end = min(a.M, s_begin + a.spc);
    const int ntiles = (s_end - s_begin) / SPT;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.in) + (long long)c * a.chan_stride +
                          ((long long)d * a.M + s_begin + lsp) * N + (long long)n1_0 * S + ln2;
    const long long tile_words = (long long)SPT * N;

    float acc[NACC];
#pragma unroll
    for (int i = 0; i < NACC; ++i) acc[i] = 0.0f;
    float2 acc2[NACC2];
#pragma unroll
    for (int i = 0; i < NACC2; ++i) acc2[i] = make_float2(0.0f, 0.0f);

    // prologue: tile 0 through stage 1 and into stage 2
    load(src);
    convert();
    if (ntiles > 1) load(src + tile_words);
    if ((stop = sync_for_mma())) break;
    if (tid == 0) issue_s1();
    wait(mb1, ph1);
    epi1();
    if ((stop = sync_for_mma())) break;
    if (tid == 0) issue_s2();

    for (int t = 0; t < ntiles; ++t) {
      const bool more = t + 1 < ntiles;
      if (more) {
        // the stage-1 MMAs of tile t have completed: their operand is free
        convert();
        if (t + 2 < ntiles) load(src + (t + 2) * tile_words);
        if ((stop = sync_for_mma())) break;
        if (tid == 0) issue_s1();
      }
      wait(mb2, ph2);
      epi2(acc, acc2);
      if (more) {
        wait(mb1, ph1);
        epi1();
        if ((stop = sync_for_mma())) break;
        if (tid == 0) issue_s2();
      }
    }
    if (stop) break;

    // ---- the unit's (chunk's) spectrum: fixed-order sum over the tile's sequences
    if ((stop = __syncthreads_or(bad) != 0)) break;
    // bin k1 + S k2 of this thread: k2 = 8 (2 qq + half) + i for its acc[8 qq + i]
    if constexpr (POL == POL_TP) {
#pragma unroll
      for (int j = 0; j < S / 2; ++j)
        red[seq * N + r + S * (8 * (2 * (j / 8) + half) + j % 8)] = acc2[j].x + acc2[j].y;
    } else {
      const int sp = seq >> 1, pl = seq & 1;
#pragma unroll
      for (int j = 0; j < S / 2; ++j) {
        const int k2 = 8 * (2 * (j / 8) + half) + j % 8;
        red[(pl * SPT + sp) * N + r + S * k2] = acc[j];
        red[((pl + 2) * SPT + sp) * N + r + S * k2] = acc[S / 2 + j];
      }
    }
    __syncthreads();
    for (int o = tid; o < NP * N; o += T) {
      const int pl = o / N, k = o - pl * N;
      float s = 0.0f;
      if constexpr (POL == POL_TP) {
#pragma unroll
        for (int q = 0; q < NSEQ; ++q) s += red[q * N + k];
      } else {
#pragma unroll
        for (int sp = 0; sp < SPT; ++sp) s += red[(pl * SPT + sp) * N + k];
      }
      if (a.chunks > 1) {
        a.partial[(((size_t)unit * a.chunks + chunk) * NP + pl) * N + k] = s;
      } else {
        float* dst = a.out + (((size_t)d * NP + pl) * a.Nc + c) * N + out_pos(k, N, a.inverse);
        if (a.mode == ACC_ADD) *dst = __fmaf_rn(s, a.scale, *dst); else *dst = s * a.scale;
      }
    }
    __syncthreads();
  }

  // No MMA is still running when the tensor memory is freed: after a normal
  // run every commit has been waited for; after a time-out the issuing
  // thread waits (bounded) for the last commit of each barrier (the phases
  // of an mbarrier complete in order).  Every tensor-memory load has
  // completed (tcgen05.wait::ld) as well.
  if (tid == 0) {
    if (ncommit[0] > 0 && !tc::mbar_wait_bounded(mb1, (ncommit[0] - 1) & 1u, kTcWaitCycles)) bad = 1;
    if (ncommit[1] > 0 && !tc::mbar_wait_bounded(mb2, (ncommit[1] - 1) & 1u, kTcWaitCycles)) bad = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
  if (bad) atomicExch(a.err, 1);
}

// Plan-time tables in the byte layout of the kernel's shared memory: the DFT
// operand (rows [hi | lo] x (k, re/im), columns (n, re/im); FP64 sincospi,
// hi = FP16(w), lo = FP16(w - hi)) and the twiddles W_N^(n2 k1) as [k1][n2].
template <int S>
__global__ void k_tc_tables(unsigned char* tab) {
  using C = TcCfg<S>;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < C::ND * C::K) {
    const int j = i / C::K, kk = i % C::K;
    const int h = j / (2 * S), k = (j % (2 * S)) >> 1, cc = j & 1, n = kk >> 1, dd = kk & 1;
    double sn, cs;
    sincospi(2.0 * ((n * k) % S) / S, &sn, &cs);
    // W = cs - i sn;  (xr + i xi) W = (xr cs + xi sn) + i (xi cs - xr sn)
    const double v = cc == 0 ? (dd == 0 ? cs : sn) : (dd == 0 ? -sn : cs);
    const __half hv = __double2half(v);
    const __half out = h == 0 ? hv : __double2half(v - (double)__half2float(hv));
    *reinterpret_cast<__half*>(tab + (j >> 3) * C::SBO + (kk >> 3) * C::LBO + (j & 7) * 16 + (kk & 7) * 2) = out;
  }
  if (i < C::N) {
    const int k1 = i / S, n2 = i % S;
    double sn, cs;
    sincospi(2.0 * (k1 * n2) / C::N, &sn, &cs);
    reinterpret_cast<float2*>(tab + C::B_BYTES)[i] = make_float2((float)cs, (float)-sn);
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

// op: 0 launch, 1 allow the dynamic shared memory, 2 also report the
// resident CTAs per SM in *occ.
template <int S, int POL>
cudaError_t tc_launch_t(const TcLaunch& L, cudaStream_t s, int op, int* occ) {
  auto k = k_tc<S, POL>;
  constexpr int smem = TcCfg<S>::SMEM;
  if (op != 0) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    // the whole unified L1/shared array as shared memory, so that the
    // occupancy query (and the launch) count on the largest carveout
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k, cudaFuncAttributePreferredSharedMemoryCarveout, cudaSharedmemCarveoutMaxShared);
    if (e != cudaSuccess || op == 1) return e;
    // resident CTAs per SM from the kernel's registers and shared memory
    // (computed here: the occupancy query reports one CTA per SM for this
    // kernel, where the hardware places two)
    cudaFuncAttributes fa;
    int dev = 0, regs_sm = 0, smem_sm = 0, smem_rsv = 0;
    if ((e = cudaFuncGetAttributes(&fa, k)) != cudaSuccess || (e = cudaGetDevice(&dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&regs_sm, cudaDevAttrMaxRegistersPerMultiprocessor, dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&smem_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev)) != cudaSuccess ||
        (e = cudaDeviceGetAttribute(&smem_rsv, cudaDevAttrReservedSharedMemoryPerBlock, dev)) != cudaSuccess)
      return e;
    const int regs_cta = ((fa.numRegs + 7) / 8 * 8) * TcCfg<S>::THREADS;
    *occ = std::min(regs_sm / std::max(regs_cta, 1), smem_sm / (smem + smem_rsv));
    return cudaSuccess;
  }
  const int items = L.unit_count * L.chunks;
  const int grid = std::min(items, std::max(L.slots, 1));
  if (grid < 1) return cudaSuccess;
  k<<<grid, TcCfg<S>::THREADS, smem, s>>>(L);
  return cudaGetLastError();
}

template <int S>
cudaError_t tc_pol(const TcLaunch& L, cudaStream_t s, int op, int* occ) {
  if (L.pol == POL_TP) return tc_launch_t<S, POL_TP>(L, s, op, occ);
  if constexpr (S <= 32) {
    if (L.pol == POL_FULL) return tc_launch_t<S, POL_FULL>(L, s, op, occ);
    if (L.pol == POL_STOKES) return tc_launch_t<S, POL_STOKES>(L, s, op, occ);
  }
  return cudaErrorInvalidValue;
}

cudaError_t tc_dispatch(const TcLaunch& L, cudaStream_t s, int op, int* occ = nullptr) {
  switch (L.logN) {
    case 8: return tc_pol<16>(L, s, op, occ);
    case 10: return tc_pol<32>(L, s, op, occ);
    case 12: return tc_pol<64>(L, s, op, occ);
    default: return cudaErrorInvalidValue;
  }
}

int tc_side(int logN) { return 1 << (logN / 2); }

// Spectra per chunk (a multiple of the spectra per tile) for `units` units
// of M spectra on `slots` resident CTAs: the CTAs take the (unit, chunk)
// items in turn, so the split that keeps the last round fullest wins.
int tc_spc(int M, int spt, int units, int slots) {
  const int max_chunks = std::max(1, M / spt);
  auto actual = [&](int c) {
    const int spc = ((M + c - 1) / c + spt - 1) / spt * spt;
    return (M + spc - 1) / spc;
  };
  auto eff = [&](int c) {
    const double items = (double)units * actual(c);
    return items / (slots * std::ceil(items / slots));
  };
  int best = 1;
  const int cap = std::min(max_chunks, std::max(1, 2 * ((slots + units - 1) / units)));
  for (int c = 2; c <= cap; ++c)
    if (eff(c) > eff(best) + 0.01) best = c;
  return ((M + best - 1) / best + spt - 1) / spt * spt;
}

}  // namespace

bool tc_supported(int logN, int fmt, int nv, int pol, int M) {
  if (logN <= 5) return tcs_supported(logN, fmt, nv, pol, M);
  if (fmt != FMT_I8 || nv != 2) return false;
  if (logN != 8 && logN != 10 && logN != 12) return false;
  if (logN == 12 && pol != POL_TP) return false;
  return M % (64 / tc_side(logN)) == 0;
}

size_t tc_table_bytes(int logN) {
  if (logN <= 5) return tcs_table_bytes(logN);
  switch (logN) {
    case 8: return TcCfg<16>::TAB_BYTES;
    case 10: return TcCfg<32>::TAB_BYTES;
    case 12: return TcCfg<64>::TAB_BYTES;
    default: return 0;
  }
}

cudaError_t tc_table_fill(void* dst, int logN, cudaStream_t s) {
  const size_t bytes = tc_table_bytes(logN);
  if (!bytes) return cudaErrorInvalidValue;
  cudaError_t e = cudaMemsetAsync(dst, 0, bytes, s);
  if (e != cudaSuccess) return e;
  if (logN <= 5) return tcs_table_fill(dst, logN, s);
  unsigned char* t = static_cast<unsigned char*>(dst);
  switch (logN) {
    case 8: k_tc_tables<16><<<(TcCfg<16>::ND * TcCfg<16>::K + 255) / 256, 256, 0, s>>>(t); break;
    case 10: k_tc_tables<32><<<(TcCfg<32>::ND * TcCfg<32>::K + 255) / 256, 256, 0, s>>>(t); break;
    default: k_tc_tables<64><<<(TcCfg<64>::ND * TcCfg<64>::K + 255) / 256, 256, 0, s>>>(t); break;
  }
  return cudaGetLastError();
}

int tc_configure(TcLaunch& L, size_t* partial_floats, int pipe_groups) {
  if (L.M < 1 || L.n_units < 1) return -1;
  int occ = 0, sms = 0, dev = 0, spt = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
      cudaSuccess)
    return -1;
  if (L.logN <= 5) {  // one-stage kernel k_tcs: 64 spectra per tile
    size_t smem = 0;
    if (tcs_plan(L, &occ, &smem) != cudaSuccess || occ < 1) return -1;
    spt = 64;
    L.smem = smem;
  } else {
    if (tc_dispatch(L, nullptr, 2, &occ) != cudaSuccess || occ < 1) return -1;
    const int S = tc_side(L.logN);
    spt = 64 / S;
    occ = std::min(occ, 512 / (8 * S));  // tensor-memory columns of the SM
    L.smem = (L.logN == 8) ? TcCfg<16>::SMEM : (L.logN == 10) ? TcCfg<32>::SMEM : TcCfg<64>::SMEM;
  }
  L.slots = occ * sms;
  L.spc = tc_spc(L.M, spt, L.n_units, L.slots);
  L.chunks = (L.M + L.spc - 1) / L.spc;
  const int gunits = std::max(1, L.n_units / std::max(1, pipe_groups));
  L.spc_pipe = tc_spc(L.M, spt, gunits, L.slots);
  L.chunks_pipe = (L.M + L.spc_pipe - 1) / L.spc_pipe;
  const int cmax = std::max(L.chunks, L.chunks_pipe);
  const int np = L.pol == POL_TP ? 1 : 4;
  *partial_floats = cmax > 1 ? (size_t)L.n_units * cmax * np * ((size_t)1 << L.logN) : 0;
  L.unit0 = 0;
  L.unit_count = L.n_units;
  if (getenv("RAWSPEC_GB300_VERBOSE"))
    fprintf(stderr, "k_tc: N %d, pol %d, units %d x %d spectra, %d resident CTAs (%d per SM), %d chunks of %d "
                    "spectra (%d of %d per channel group)\n", 1 << L.logN, L.pol, L.n_units, L.M, L.slots, occ,
            L.chunks, L.spc, L.chunks_pipe, L.spc_pipe);
  return 0;
}

cudaError_t tc_launch(const TcLaunch& L, cudaStream_t s) {
  return L.logN <= 5 ? tcs_launch(L, s) : tc_dispatch(L, s, 0);
}

}  // namespace rsg
