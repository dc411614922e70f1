// k_small.cu -- fused spectrometer kernel for FFT lengths N <= 4096.
//
// One launch per output product and input buffer replaces the reference's
// per-(product, batch, pol) cufftExecC2C calls with their texture load
// callback and read-modify-write store callbacks (rawspec_gpu.cu:1555-1569,
// :133-267), the sub-integration `accumulate` kernel (:297-318, :1588-1601)
// and the FFT-shifting device-to-host copies (:1647-1697):
//
//   int8/int16 load + exact integer unpack -> Stockham FFT in registers and
//   shared memory (both polarisations together) -> detection -> accumulation
//   of the unit's spectra in registers -> reduction across the CTA's thread
//   groups -> SNORM scale and FFT-shifted store into the dump buffer
//   [Nd][|P|][Nc][N] (or partial sums when one unit is spread over CTAs).
//
// Nothing but the raw voltages is read and nothing but integrated spectra is
// written.
#include <algorithm>
#include <cmath>

#include "detect.cuh"
#include "fft_core.cuh"
#include "internal.h"

namespace rsg {

// R (values per thread per polarisation) is 16 for total power and 8 for the
// four-plane modes, whose 4*R accumulators would otherwise not fit the
// register cap of two resident CTAs per SM.
template <int N, int NP>
struct SmallCfg {
  static constexpr int RMAX = NP == 1 ? 16 : 8;
  static constexpr int R = N < RMAX ? N : RMAX;
  static constexpr int T = N / R;            // threads per FFT
  static constexpr int TPB = T > 256 ? T : 256;
  static constexpr int G = TPB / T;          // FFT groups per CTA
  static constexpr int MINB = 65536 / (TPB * 128) > 0 ? 65536 / (TPB * 128) : 1;
  static constexpr int TW = stockham_tw_size(N, R);  // twiddle table entries
};

struct WarpSync {
  __device__ __forceinline__ void operator()() const { __syncwarp(); }
};
// Barrier of one transform group that spans whole warps (named barrier
// 1 + group, `threads` = the group's thread count), so that the groups of a
// CTA progress independently.
struct GroupSync {
  int id, threads;
  __device__ __forceinline__ void operator()() const {
    asm volatile("bar.sync %0, %1;" ::"r"(id), "r"(threads) : "memory");
  }
};

// Floats between the groups' slices of the reduction area: the slice
// (NP R T floats) padded so that, with T < 32 threads per group, the groups
// of a warp start T banks apart and their writes fall into distinct banks.
template <int N, int NP>
__host__ __device__ constexpr int small_red_stride() {
  using C = SmallCfg<N, NP>;
  constexpr int rb = NP * C::R * C::T;
  return C::T >= 32 ? rb : rb + ((C::T - rb % 32) % 32 + 32) % 32;
}

template <int N, int NV, int NP>
__host__ __device__ constexpr size_t small_smem_bytes() {
  using C = SmallCfg<N, NP>;
  const size_t tw = (size_t)((C::TW + 1) & ~1) * sizeof(float2);
  const size_t xch = (C::T > 1) ? (size_t)C::G * NV * smem_padded_len(N) * sizeof(float2) : 0;
  const size_t red = (size_t)C::G * small_red_stride<N, NP>() * sizeof(float);
  return tw + (xch > red ? xch : red);
}

// The kernel body for CTA `bid` of launch `a` (k_small: one launch;
// k_small_group: several launches of the same configuration, e.g. the
// buffers of several jobs, in one grid).
template <int N, int FMT, int NV, int POL>
__device__ __forceinline__ void small_body(const SmallLaunch& a, const int bid) {
  constexpr int NP = PolOut<POL>::NP;
  using C = SmallCfg<N, NP>;
  constexpr int R = C::R, T = C::T, G = C::G, TPB = C::TPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];

  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* xch = tw_s + ((C::TW + 1) & ~1);
  float* red = reinterpret_cast<float*>(xch);

  const int tid = threadIdx.x;
  const int g = tid / T;   // group within the CTA
  const int j = tid % T;   // thread within the group

  if constexpr (C::TW > 0) {
    for (int i = tid; i < C::TW; i += TPB) tw_s[i] = a.tw[i];
    __syncthreads();
  }

  // Which unit / spectra this group works on.  The CTA covers `sets` units
  // (gps groups each) and one chunk of spc spectra of each of them.
  const int gps = G / a.sets;           // groups per set
  const int set = g / gps;
  const int gi = g % gps;
  const int ublock = bid / a.chunks;
  const int chunk = bid % a.chunks;
  const int unit = a.unit0 + ublock * a.sets + set;
  const int s_begin = chunk * a.spc;
  const int s_end = min(a.M, s_begin + a.spc);
  const bool unit_ok = unit < a.unit0 + a.unit_count;
  const int c = unit_ok ? unit / a.units_per_chan : 0;
  const int d = unit_ok ? unit % a.units_per_chan : 0;
  const long long chan_base = (long long)c * a.chan_stride;
  const long long unit_first_spec = (long long)d * a.M;
  const int iters = (a.spc + gps - 1) / gps;
  const float im_sign = a.conj ? -1.0f : 1.0f;

  float acc[R][NP];
#pragma unroll
  for (int m = 0; m < R; ++m)
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[m][p] = 0.0f;
  // Total power of two polarisations on the packed instructions: one lane
  // per polarisation, the lanes summed after the last spectrum.
  constexpr bool kPackedTP = POL == POL_TP && NV == 2 && RSG_PACKED;
  // Cross products of two polarisations: the two powers as one packed pair
  // (|X0|^2, |X1|^2), the cross terms Re and Im(X0 X1*) unsigned; Stokes I
  // and Q and the conjugation sign are linear in these sums and applied
  // after the last spectrum.
  constexpr bool kPackedX = POL != POL_TP && NV == 2 && RSG_PACKED;
  float2 acc2[(kPackedTP || kPackedX) ? R : 1];
#pragma unroll
  for (int m = 0; m < ((kPackedTP || kPackedX) ? R : 1); ++m) acc2[m] = make_float2(0.f, 0.f);

  float2* my_xch = xch + (size_t)g * NV * smem_padded_len(N);

  using W = typename SampleWord<FMT, NV>::type;
  constexpr bool kVec = T == 1 && (R * sizeof(W)) % 16 == 0;
  // Words of spectrum `it` of this group (zeros past the unit's end).
  auto load_words = [&](int it, W (&w)[R]) {
    const int s_local = s_begin + gi + it * gps;
    if (!(unit_ok && s_local < s_end)) {
#pragma unroll
      for (int m = 0; m < R; ++m) w[m] = W{};
      return;
    }
    const W* src = reinterpret_cast<const W*>(a.in) + chan_base + (unit_first_spec + s_local) * N + j;
    if (kVec && a.vec16) {
      // one thread per transform: its R contiguous words in 16-byte loads
      const uint4* s4 = reinterpret_cast<const uint4*>(src);
#pragma unroll
      for (int i = 0; i < (int)(R * sizeof(W) / 16); ++i) {
        const uint4 u = __ldg(s4 + i);
        memcpy(reinterpret_cast<char*>(w) + 16 * i, &u, 16);
      }
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m) w[m] = __ldg(src + m * T);
    }
  };
  // The next spectrum's words are requested before the current transform
  // when the registers allow it (spectra of one thread, or 8 values per
  // thread); otherwise each spectrum is loaded when it is processed.
  constexpr bool kPrefetch = T == 1 || (NV == 2 ? R <= 8 : R <= 16);
  static_assert(kPrefetch || !kVec, "vector loads only on the prefetching path");
  W wn[kPrefetch ? R : 1];
  if constexpr (kPrefetch) load_words(0, wn);

  for (int it = 0; it < iters; ++it) {
    const int s_local = s_begin + gi + it * gps;
    const bool valid = unit_ok && s_local < s_end;
    float2 v[NV][R];
    if constexpr (kPrefetch) {
      W w[R];
#pragma unroll
      for (int m = 0; m < R; ++m) w[m] = wn[m];
      if (it + 1 < iters) load_words(it + 1, wn);
#pragma unroll
      for (int m = 0; m < R; ++m) {
        float2 smp[NV];
        Unpack<FMT, NV>::run(w[m], smp);
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q][m] = smp[q];
      }
    } else if (valid) {
      const W* src = reinterpret_cast<const W*>(a.in) + chan_base + (unit_first_spec + s_local) * N + j;
      W w[R];
#pragma unroll
      for (int m = 0; m < R; ++m) w[m] = __ldg(src + m * T);
#pragma unroll
      for (int m = 0; m < R; ++m) {
        float2 smp[NV];
        Unpack<FMT, NV>::run(w[m], smp);
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q][m] = smp[q];
      }
    } else {
#pragma unroll
      for (int m = 0; m < R; ++m)
#pragma unroll
        for (int q = 0; q < NV; ++q) v[q][m] = make_float2(0.f, 0.f);
    }
    if constexpr (T > 32) {
      static_assert(G <= 15, "one named barrier per group");
      GroupFFT<N, R, NV>::run(v, j, my_xch, smem_padded_len(N), tw_s, GroupSync{1 + g, T});
    } else {
      GroupFFT<N, R, NV>::run(v, j, my_xch, smem_padded_len(N), tw_s, WarpSync{});
    }
    if (valid) {
      if constexpr (kPackedTP) {
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const cpair x = pack2(v[0][m], v[1][m]);
          acc2[m] = f2fma(x.im, x.im, f2fma(x.re, x.re, acc2[m]));
        }
      } else if constexpr (kPackedX) {
#pragma unroll
        for (int m = 0; m < R; ++m) {
          const float2 x0 = v[0][m], x1 = v[1][m];
          const cpair x = pack2(x0, x1);
          acc2[m] = f2fma(x.im, x.im, f2fma(x.re, x.re, acc2[m]));
          acc[m][2] = __fmaf_rn(x0.y, x1.y, __fmaf_rn(x0.x, x1.x, acc[m][2]));
          acc[m][3] = __fmaf_rn(-x0.x, x1.y, __fmaf_rn(x0.y, x1.x, acc[m][3]));
        }
      } else {
#pragma unroll
        for (int m = 0; m < R; ++m) {
          float2 x[NV];
#pragma unroll
          for (int q = 0; q < NV; ++q) x[q] = v[q][m];
          detect_acc<POL, NV>(acc[m], x, im_sign);
        }
      }
    }
  }
  if constexpr (kPackedTP) {
#pragma unroll
    for (int m = 0; m < R; ++m) acc[m][0] = acc2[m].x + acc2[m].y;
  }
  if constexpr (kPackedX) {
#pragma unroll
    for (int m = 0; m < R; ++m) {
      if constexpr (POL == POL_FULL) {
        acc[m][0] = acc2[m].x;
        acc[m][1] = acc2[m].y;
      } else {
        acc[m][0] = acc2[m].x + acc2[m].y;
        acc[m][1] = acc2[m].x - acc2[m].y;
      }
      acc[m][3] *= im_sign;
    }
  }

  // Reduce across the groups of each set: red[g][p][m][j], the groups'
  // slices padded apart (small_red_stride) so that their writes fall into
  // different banks (with one thread per transform they would all hit one).
  constexpr int RS = small_red_stride<N, NP>();
  __syncthreads();
#pragma unroll
  for (int p = 0; p < NP; ++p)
#pragma unroll
    for (int m = 0; m < R; ++m) red[g * RS + (p * R + m) * T + j] = acc[m][p];
  __syncthreads();

  const int set_threads = gps * T;
  const int t_in_set = tid - set * set_threads;
  if (!unit_ok) return;
  for (int o = t_in_set; o < NP * N; o += set_threads) {
    const int p = o / N;
    const int k = o - p * N;
    const int m = k / T;
    const int jj = k - m * T;
    float s = 0.0f;
    for (int q = 0; q < gps; ++q) s += red[(set * gps + q) * RS + (p * R + m) * T + jj];
    if (a.chunks > 1) {
      a.partial[(((size_t)unit * a.chunks + chunk) * NP + p) * N + k] = s;
    } else {
      float* dst = a.out + (((size_t)d * NP + p) * a.Nc + c) * N + out_pos(k, N, a.inverse);
      if (a.mode == ACC_ADD) *dst = __fmaf_rn(s, a.scale, *dst); else *dst = s * a.scale;
    }
  }
}

template <int N, int FMT, int NV, int POL>
__global__ void __launch_bounds__(SmallCfg<N, PolOut<POL>::NP>::TPB, SmallCfg<N, PolOut<POL>::NP>::MINB)
k_small(const __grid_constant__ SmallLaunch a) {
  small_body<N, FMT, NV, POL>(a, blockIdx.x);
}

// Several launches of one configuration in one grid: CTA b belongs to the
// launch k whose range [end[k-1], end[k]) holds it.
template <int N, int FMT, int NV, int POL>
__global__ void __launch_bounds__(SmallCfg<N, PolOut<POL>::NP>::TPB, SmallCfg<N, PolOut<POL>::NP>::MINB)
k_small_group(const __grid_constant__ SmallGroup g) {
  int k = 0;
  while (k + 1 < g.n && (int)blockIdx.x >= g.end[k]) ++k;
  small_body<N, FMT, NV, POL>(g.e[k], (int)blockIdx.x - (k ? g.end[k - 1] : 0));
}

// Finalisation of chunked units: fixed-order sum of the chunks' partials,
// SNORM scale and FFT-shifted store.
__global__ void k_finalize(FinalizeLaunch a) {
  const long long total = (long long)a.n_units * a.np * a.N;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
       i += (long long)gridDim.x * blockDim.x) {
    const int k = (int)(i % a.N);
    const long long up = i / a.N;
    const int p = (int)(up % a.np);
    const int unit = a.unit0 + (int)(up / a.np);
    const float* src = a.partial + ((size_t)unit * a.chunks * a.np + p) * a.N + k;
    float s = 0.0f;
    for (int q = 0; q < a.chunks; ++q) s += src[(size_t)q * a.np * a.N];
    const int c = unit / a.units_per_chan;
    const int d = unit % a.units_per_chan;
    float* dst = a.out + (((size_t)d * a.np + p) * a.Nc + c) * a.N + out_pos(k, a.N, a.inverse);
    if (a.mode == ACC_ADD) *dst = __fmaf_rn(s, a.scale, *dst); else *dst = s * a.scale;
  }
}

// ---------------------------------------------------------------------------
// Host side: configuration and dispatch.
// ---------------------------------------------------------------------------
namespace {

struct SmallInfo {
  int R, T, TPB, G;
  size_t smem;
};

template <int N, int NP>
SmallInfo small_info_np(int nv) {
  using C = SmallCfg<N, NP>;
  SmallInfo s{C::R, C::T, C::TPB, C::G, 0};
  s.smem = nv == 1 ? small_smem_bytes<N, 1, NP>() : small_smem_bytes<N, 2, NP>();
  return s;
}
template <int N>
SmallInfo small_info(int nv, int pol) {
  return pol == POL_TP ? small_info_np<N, 1>(nv) : small_info_np<N, 4>(nv);
}

SmallInfo small_info_dyn(int logN, int nv, int pol) {
  switch (logN) {
    case 0: return small_info<1>(nv, pol);
    case 1: return small_info<2>(nv, pol);
    case 2: return small_info<4>(nv, pol);
    case 3: return small_info<8>(nv, pol);
    case 4: return small_info<16>(nv, pol);
    case 5: return small_info<32>(nv, pol);
    case 6: return small_info<64>(nv, pol);
    case 7: return small_info<128>(nv, pol);
    case 8: return small_info<256>(nv, pol);
    case 9: return small_info<512>(nv, pol);
    case 10: return small_info<1024>(nv, pol);
    case 11: return small_info<2048>(nv, pol);
    default: return small_info<4096>(nv, pol);
  }
}

int small_grid(const SmallLaunch& L) { return ((L.unit_count + L.sets - 1) / L.sets) * L.chunks; }

// op: 0 launch, 1 allow the dynamic shared memory, 2 also report the
// resident CTAs per SM in *occ, 3 launch the group *grp (entries of L's
// configuration).
template <int N, int FMT, int NV, int POL>
cudaError_t launch_t(const SmallLaunch& L, cudaStream_t s, int op, int* occ, const SmallGroup* grp) {
  auto k = k_small<N, FMT, NV, POL>;
  if (op == 3) {
    auto kg = k_small_group<N, FMT, NV, POL>;
    cudaError_t e = cudaFuncSetAttribute(kg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    if (e != cudaSuccess) return e;
    const int grid = grp->end[grp->n - 1];
    if (grid < 1) return cudaSuccess;
    kg<<<grid, SmallCfg<N, PolOut<POL>::NP>::TPB, L.smem, s>>>(*grp);
    return cudaGetLastError();
  }
  if (op != 0) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L.smem);
    if (e != cudaSuccess || op == 1) return e;
    return cudaOccupancyMaxActiveBlocksPerMultiprocessor(occ, k, SmallCfg<N, PolOut<POL>::NP>::TPB, L.smem);
  }
  const int grid = small_grid(L);
  if (grid < 1) return cudaSuccess;
  k<<<grid, SmallCfg<N, PolOut<POL>::NP>::TPB, L.smem, s>>>(L);
  return cudaGetLastError();
}

template <int N, int FMT>
cudaError_t launch_pol(const SmallLaunch& L, cudaStream_t s, int op, int* occ, const SmallGroup* grp) {
  if (L.nv == 1) return launch_t<N, FMT, 1, POL_TP>(L, s, op, occ, grp);
  switch (L.pol) {
    case POL_FULL: return launch_t<N, FMT, 2, POL_FULL>(L, s, op, occ, grp);
    case POL_STOKES: return launch_t<N, FMT, 2, POL_STOKES>(L, s, op, occ, grp);
    default: return launch_t<N, FMT, 2, POL_TP>(L, s, op, occ, grp);
  }
}

template <int N>
cudaError_t launch_fmt(const SmallLaunch& L, cudaStream_t s, int op, int* occ, const SmallGroup* grp) {
  return L.fmt == FMT_I16 ? launch_pol<N, FMT_I16>(L, s, op, occ, grp) : launch_pol<N, FMT_I8>(L, s, op, occ, grp);
}

cudaError_t small_dispatch(const SmallLaunch& L, cudaStream_t s, int op, int* occ = nullptr,
                           const SmallGroup* grp = nullptr) {
  switch (L.logN) {
    case 0: return launch_fmt<1>(L, s, op, occ, grp);
    case 1: return launch_fmt<2>(L, s, op, occ, grp);
    case 2: return launch_fmt<4>(L, s, op, occ, grp);
    case 3: return launch_fmt<8>(L, s, op, occ, grp);
    case 4: return launch_fmt<16>(L, s, op, occ, grp);
    case 5: return launch_fmt<32>(L, s, op, occ, grp);
    case 6: return launch_fmt<64>(L, s, op, occ, grp);
    case 7: return launch_fmt<128>(L, s, op, occ, grp);
    case 8: return launch_fmt<256>(L, s, op, occ, grp);
    case 9: return launch_fmt<512>(L, s, op, occ, grp);
    case 10: return launch_fmt<1024>(L, s, op, occ, grp);
    case 11: return launch_fmt<2048>(L, s, op, occ, grp);
    case 12: return launch_fmt<4096>(L, s, op, occ, grp);
    default: return cudaErrorInvalidValue;
  }
}

// Chunks per unit: at least c_min (the parallelism asked for), raised while
// that makes the grid fill its last wave of resident CTAs markedly better
// (all CTAs of a launch take about the same time, so a grid of 2.1 waves
// runs as long as one of 3).  Units processed whole (c_min = 1) stay whole:
// splitting them would add a finalisation pass.
#ifndef RSG_SMALL_WAVEFIT
#define RSG_SMALL_WAVEFIT 1
#endif
int fit_chunks(int M, int ublocks, int c_min, int max_chunks, int slots) {
  auto actual = [&](int c) { const int spc = (M + c - 1) / c; return (M + spc - 1) / spc; };
  auto eff = [&](int c) {
    const double w = (double)ublocks * actual(c) / slots;
    return w / std::ceil(w);
  };
  int best = std::max(1, std::min(c_min, max_chunks));
  if (!RSG_SMALL_WAVEFIT || slots <= 0 || best == 1) return best;
  for (int c = best + 1; c <= std::min(max_chunks, 2 * best); ++c)
    if (eff(c) > eff(best) + 0.05) best = c;
  return best;
}

}  // namespace

int small_radix(int logN, int pol) { return small_info_dyn(logN, 2, pol).R; }

int small_configure(SmallLaunch& L, int target_ctas, size_t* partial_floats, int pipe_groups) {
  if (L.logN < 0 || L.logN > 12 || L.M < 1 || L.n_units < 1) return -1;
  const SmallInfo si = small_info_dyn(L.logN, L.nv, L.pol);
  L.tpb = si.TPB;
  L.smem = si.smem;
  const int G = si.G;
  const int np = L.pol == POL_TP ? 1 : 4;
  auto pow2_floor = [](int x) { int p = 1; while (p * 2 <= x) p *= 2; return p; };
  // Groups per unit: at most one per spectrum, and few enough that every
  // thread of a set has an output to reduce (gps <= |P| * R).
  int gps = std::min(G, std::min(pow2_floor(np * si.R), pow2_floor(L.M)));
  L.sets = G / gps;
  const int ublocks = (L.n_units + L.sets - 1) / L.sets;
  const int max_chunks = (L.M + gps - 1) / gps;
  // resident CTAs on the device
  int occ = 0, sms = 0, dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) !=
      cudaSuccess || small_dispatch(L, nullptr, 2, &occ) != cudaSuccess)
    occ = 0;
  const int slots = occ * sms;
  const int chunks = fit_chunks(L.M, ublocks, (target_ctas + ublocks - 1) / ublocks, max_chunks, slots);
  L.spc = (L.M + chunks - 1) / chunks;
  L.chunks = (L.M + L.spc - 1) / L.spc;
  L.grid = ublocks * L.chunks;
  // the same for a launch over 1/pipe_groups of the units
  {
    const int gunits = std::max(1, L.n_units / std::max(1, pipe_groups));
    const int gublocks = (gunits + L.sets - 1) / L.sets;
    const int c2 = fit_chunks(L.M, gublocks, (target_ctas + gublocks - 1) / gublocks, max_chunks, slots);
    L.spc_pipe = (L.M + c2 - 1) / c2;
    L.chunks_pipe = (L.M + L.spc_pipe - 1) / L.spc_pipe;
  }
  const int cmax = std::max(L.chunks, L.chunks_pipe);
  *partial_floats = cmax > 1 ? (size_t)L.n_units * cmax * np * ((size_t)1 << L.logN) : 0;
  L.unit0 = 0;
  L.unit_count = L.n_units;
  const long long wbytes = (L.fmt == FMT_I16 ? 4 : 2) * L.nv;
  L.vec16 = ((L.chan_stride * wbytes) % 16 == 0) && ((reinterpret_cast<uintptr_t>(L.in) & 15) == 0);
  return 0;
}

cudaError_t small_prepare(const SmallLaunch& L) { return small_dispatch(L, nullptr, 1); }
cudaError_t small_launch(const SmallLaunch& L, cudaStream_t s) { return small_dispatch(L, s, 0); }

bool small_same_kernel(const SmallLaunch& a, const SmallLaunch& b) {
  return a.logN == b.logN && a.fmt == b.fmt && a.nv == b.nv && (a.nv == 1 || a.pol == b.pol) && a.smem == b.smem;
}

cudaError_t small_launch_group(const SmallLaunch* L, int n, cudaStream_t s) {
  if (n < 1 || n > kSmallGroupMax) return cudaErrorInvalidValue;
  SmallGroup g;
  g.n = n;
  int end = 0;
  for (int k = 0; k < n; ++k) {
    if (!small_same_kernel(L[0], L[k])) return cudaErrorInvalidValue;
    g.e[k] = L[k];
    end += std::max(0, small_grid(L[k]));
    g.end[k] = end;
  }
  return small_dispatch(L[0], s, 3, nullptr, &g);
}

cudaError_t finalize_launch(const FinalizeLaunch& L, cudaStream_t s) {
  const long long total = (long long)L.n_units * L.np * L.N;
  int blocks = (int)std::min<long long>((total + 255) / 256, 152LL * 16);
  if (blocks < 1) blocks = 1;
  k_finalize<<<blocks, 256, 0, s>>>(L);
  return cudaGetLastError();
}

}  // namespace rsg
