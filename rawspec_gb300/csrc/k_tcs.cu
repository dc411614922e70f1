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
// A CTA (4 warps, one thread per tensor-memory lane) works through tiles of
// 64 spectra of one integration unit, two tiles in flight: the MMAs of tile
// t run while tile t-1 is detected.  Each thread accumulates its lane's
// powers over the unit's tiles in registers; at the end of the unit the
// lanes and warps are summed in a fixed order and the FFT-shifted spectrum
// is stored (or a partial sum per chunk of the unit, finished by
// k_finalize).
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
  static constexpr int THREADS = 128;        // one thread per tensor-memory lane
  static constexpr int SPT = 64;             // spectra per tile (x 2 polarisations = 128 rows)
  static constexpr int ACC_COLS = ND < 32 ? 32 : ND;  // tensor-memory columns per accumulator
  static constexpr int TMEM_COLS = 2 * ACC_COLS;      // two tiles in flight
  // data operands x 2 | DFT operand | 2 mbarriers, tensor-memory slot, 2 commit counters
  static constexpr int SMEM = 2 * A_BYTES + B_BYTES + 32;
  static_assert(N % 8 == 0 && N <= 32, "lengths 8, 16, 32");
  static_assert(4 * 4 * N * (int)sizeof(float) <= 2 * A_BYTES, "reduction fits the operand area");
};

namespace {

constexpr long long kTcsWaitCycles = 2000000000ll;  // ~1 s of SM clocks for a tile's MMAs

}  // namespace

template <int N, int POL>
__global__ void __launch_bounds__(TcsCfg<N>::THREADS) k_tcs(const __grid_constant__ TcLaunch a) {
  using C = TcsCfg<N>;
  constexpr int NP = PolOut<POL>::NP, SPT = C::SPT;
  constexpr uint32_t IDESC = tc::idesc_f16_f32(128, C::ND);
  // total power: (sum x^2, sum y^2) per bin on the packed instructions;
  // cross products: two planes per lane (polarisation-0 lanes planes 0 and
  // 2, polarisation-1 lanes planes 1 and 3)
  constexpr int NACC = POL == POL_TP ? N : 2 * N;
  using Acc = typename std::conditional<POL == POL_TP, float2, float>::type;
  extern __shared__ __align__(128) unsigned char sm[];
  unsigned char* sA = sm;                   // two data operands
  unsigned char* sB = sm + 2 * C::A_BYTES;  // DFT operand [hi | lo]
  uint64_t* mb = reinterpret_cast<uint64_t*>(sB + C::B_BYTES);
  uint32_t* tslot = reinterpret_cast<uint32_t*>(mb + 2);
  uint32_t* ncommit = tslot + 1;  // commits issued to mb[0] and mb[1] (thread 0)
  float* red = reinterpret_cast<float*>(sm);  // [warp][plane][bin], over the data operands

  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  {
    const uint4* src = reinterpret_cast<const uint4*>(a.tab);
    uint4* dst = reinterpret_cast<uint4*>(sB);
    for (int i = tid; i < C::B_BYTES / 16; i += C::THREADS) dst[i] = __ldg(src + i);
  }
  if (tid == 0) {
    tc::mbar_init(mb, 1);
    tc::mbar_init(mb + 1, 1);
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
  const uint32_t lane_off = (uint32_t)(warp * 32) << 16;  // this warp's lanes
  const uint32_t aA = tc::smem_u32(sA), bF = tc::smem_u32(sB), bFlo = bF + C::B_LO;
  unsigned ph = 0;  // bit b: parity of the next completion of mb[b]
  int bad = 0;      // one of this thread's waits timed out
  // row tid = polarisation pol of spectrum sp of the tile
  const int sp = tid >> 1, pol = tid & 1;
  const uint32_t sel = pol ? 0x4342u : 0x4140u;
  const float im_sign = a.conj ? -1.0f : 1.0f;

  uint4 w[N / 4];  // the spectrum's N sample words
  auto load = [&](const uint32_t* p) {
#pragma unroll
    for (int j = 0; j < N / 4; ++j) w[j] = __ldg(reinterpret_cast<const uint4*>(p) + j);
  };
  // row tid of data operand buf: samples 4c .. 4c+3 as (re, im) FP16 pairs
  // fill core matrix c of the row
  auto convert = [&](int buf) {
    unsigned char* row = sA + buf * C::A_BYTES + (tid >> 3) * C::SBO + (tid & 7) * 16;
#pragma unroll
    for (int c = 0; c < N / 4; ++c) {
      const uint32_t x[4] = {w[c].x, w[c].y, w[c].z, w[c].w};
      uint32_t h[4];
#pragma unroll
      for (int i = 0; i < 4; ++i) h[i] = tc::codes_to_h2(__vmaxs4(x[i], 0x81818181u) ^ 0x80808080u, sel);
      *reinterpret_cast<uint4*>(row + c * C::LBO) = make_uint4(h[0], h[1], h[2], h[3]);
    }
  };
  // codes x (F hi + F lo) into accumulator buf
  auto issue = [&](int buf) {
    const uint32_t d = tmem + buf * C::ACC_COLS, aa = aA + buf * C::A_BYTES;
#pragma unroll
    for (int ks = 0; ks < C::K / 16; ++ks)
      tc::mma_f16(d, tc::smem_desc(aa + ks * 2 * C::LBO, C::LBO, C::SBO),
                  tc::smem_desc(bF + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, ks > 0 ? 1u : 0u);
#pragma unroll
    for (int ks = 0; ks < C::K / 16; ++ks)
      tc::mma_f16(d, tc::smem_desc(aa + ks * 2 * C::LBO, C::LBO, C::SBO),
                  tc::smem_desc(bFlo + ks * 2 * C::LBO, C::LBO, C::SBO), IDESC, 1u);
    tc::mma_commit(mb + buf);
    ++ncommit[buf];
  };
  // waits for accumulator buf and adds its detected values
  auto detect = [&](int buf, Acc (&acc)[NACC]) {
    if (!tc::mbar_wait_bounded(mb + buf, (ph >> buf) & 1u, kTcsWaitCycles)) bad = 1;
    ph ^= 1u << buf;
    tc::fence_after_sync();
    const uint32_t d = tmem + buf * C::ACC_COLS + lane_off;
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
          const float2 Y = make_float2(__shfl_xor_sync(0xffffffffu, X.x, 1), __shfl_xor_sync(0xffffffffu, X.y, 1));
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

  const int items = a.unit_count * a.chunks;
  int buf = 0;
  bool stop = false;
  for (int item = blockIdx.x; item < items && !stop; item += gridDim.x) {
    const int unit = a.unit0 + item / a.chunks, chunk = item % a.chunks;
    const int c = unit / a.units_per_chan, d = unit % a.units_per_chan;
    const int s_begin = chunk * a.spc;
    const int s_end = min(a.M, s_begin + a.spc);
    const int ntiles = (s_end - s_begin) / SPT;
    const uint32_t* src = reinterpret_cast<const uint32_t*>(a.in) + (long long)c * a.chan_stride +
                          ((long long)d * a.M + s_begin + sp) * N;

    Acc acc[NACC];
#pragma unroll
    for (int i = 0; i < NACC; ++i) acc[i] = Acc{};

    load(src);
    for (int t = 0; t < ntiles; ++t) {
      // operand and accumulator buf were last used by tile t-2, detected
      // (its MMAs complete, its tensor-memory loads waited for) before the
      // barrier below
      convert(buf);
      if (t + 1 < ntiles) load(src + (long long)(t + 1) * SPT * N);
      tc::fence_proxy_async_smem();
      tc::fence_before_sync();
      if ((stop = __syncthreads_or(bad) != 0)) break;
      if (tid == 0) {
        tc::fence_after_sync();
        issue(buf);
      }
      if (t > 0) detect(buf ^ 1, acc);
      buf ^= 1;
    }
    if (stop) break;
    if (ntiles > 0) detect(buf ^ 1, acc);
    if ((stop = __syncthreads_or(bad) != 0)) break;

    // ---- the unit's (chunk's) spectrum: lanes, then warps, in a fixed order
    if constexpr (POL == POL_TP) {
#pragma unroll
      for (int k = 0; k < N; ++k) {
        float s = acc[k].x + acc[k].y;
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        if (lane == 0) red[warp * N + k] = s;
      }
    } else {
#pragma unroll
      for (int j = 0; j < 2 * N; ++j) {
        float s = acc[j];
#pragma unroll
        for (int off = 16; off > 1; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
        // lane 0: planes 0 (j < N) and 2; lane 1: planes 1 and 3
        if (lane < 2) red[(warp * 4 + lane + (j < N ? 0 : 2)) * N + (j % N)] = s;
      }
    }
    __syncthreads();
    for (int o = tid; o < NP * N; o += C::THREADS) {
      const int pl = o / N, k = o - pl * N;
      float s = 0.0f;
#pragma unroll
      for (int wq = 0; wq < 4; ++wq) s += red[(wq * NP + pl) * N + k];
      if (a.chunks > 1) {
        a.partial[(((size_t)unit * a.chunks + chunk) * NP + pl) * N + k] = s;
      } else {
        float* dst = a.out + (((size_t)d * NP + pl) * a.Nc + c) * N + out_pos(k, N, a.inverse);
        if (a.mode == ACC_ADD) *dst = __fmaf_rn(s, a.scale, *dst); else *dst = s * a.scale;
      }
    }
    __syncthreads();  // the reduction area is the next unit's data operands
  }

  // No MMA is still running when the tensor memory is freed: after a normal
  // run every commit has been waited for; after a time-out the issuing
  // thread waits (bounded) for the last commit of each barrier.
  if (tid == 0) {
    for (int b = 0; b < 2; ++b)
      if (ncommit[b] > 0 && !tc::mbar_wait_bounded(mb + b, (ncommit[b] - 1) & 1u, kTcsWaitCycles)) bad = 1;
  }
  tc::fence_before_sync();
  __syncthreads();
  tc::fence_after_sync();
  if (warp == 0) tc::tmem_dealloc(tmem, C::TMEM_COLS);
  if (bad) atomicExch(a.err, 1);
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

// Resident CTAs per SM: registers, and the tensor-memory columns of the SM
// (the dynamic shared memory is padded so that no more CTAs than that fit).
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
  const int o = std::max(1, std::min(regs_sm / std::max(regs_cta, 1), 512 / C::TMEM_COLS));
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
