// k_large.cu -- four-step FFT spectrometer for 4096 < N <= 2^24.
//
// Replaces the reference's cuFFT plan for long transforms (one
// cufftExecC2C per product, channel batch and polarisation with load/store
// callbacks, rawspec_gpu.cu:1182-1195, :1555-1569) by two kernels:
//
//   pass A  N2-point FFTs down the columns of x[n1 + N1*n2] (both
//           polarisations), twiddled by W_N^(n1*k2), written to scratch as
//           [slab][pol][k2][n1] -- the only intermediate that touches global
//           memory;
//   pass B  N1-point FFTs along the rows k2 of that scratch, detection of
//           the output bins X[k2 + N2*k1], integration over the unit's
//           spectra in registers and the FFT-shifted store (or add).
//
// X[k2 + N2 k1] = sum_n1 W_N1^(n1 k1) W_N^(n1 k2) sum_n2 x[n1 + N1 n2] W_N2^(n2 k2).
#include <algorithm>

#include "detect.cuh"
#include "fft_core.cuh"
#include "internal.h"

namespace rsg {

namespace {

constexpr int kLargeR = 8;
constexpr int kLargeTPB = 512;

template <int NSUB>
struct LargeCfg {
  static constexpr int R = kLargeR;
  static constexpr int T = NSUB / R;              // threads per sub-FFT
  static constexpr int C = kLargeTPB / T > 8 ? 8 : (kLargeTPB / T > 0 ? kLargeTPB / T : 1);
  static constexpr int TPB = T * C;
};

struct BlockSyncL {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

template <int N2, int NV>
constexpr size_t passA_smem(int h, int logN) {
  using Cf = LargeCfg<N2>;
  return (size_t)N2 * sizeof(float2) + (size_t)Cf::C * NV * smem_padded_len(N2) * sizeof(float2) +
         ((size_t)1 << h) * sizeof(float2) + ((size_t)1 << (logN - h)) * sizeof(float2);
}

template <int N1, int NV>
constexpr size_t passB_smem() {
  using Cf = LargeCfg<N1>;
  return (size_t)N1 * sizeof(float2) + (size_t)Cf::C * NV * smem_padded_len(N1) * sizeof(float2);
}

}  // namespace

template <int N2, int FMT, int NV>
__global__ void __launch_bounds__(LargeCfg<N2>::TPB)
k_large_a(LargeLaunch a) {
  using Cf = LargeCfg<N2>;
  constexpr int R = Cf::R, T = Cf::T, C = Cf::C, TPB = Cf::TPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* xch = tw_s + N2;
  float2* lo_s = xch + (size_t)C * NV * smem_padded_len(N2);
  const int nlo = 1 << a.h;
  const int nhi = 1 << (a.logN - a.h);
  float2* hi_s = lo_s + nlo;

  const int tid = threadIdx.x;
  for (int i = tid; i < N2; i += TPB) tw_s[i] = a.twN2[i];
  for (int i = tid; i < nlo; i += TPB) lo_s[i] = a.twLo[i];
  for (int i = tid; i < nhi; i += TPB) hi_s[i] = a.twHi[i];
  __syncthreads();

  const int N1 = 1 << a.logN1;
  const int tiles = N1 / C;
  const int tile = blockIdx.x % tiles;
  const int slab = blockIdx.x / tiles;
  const int c = slab / a.Nss;
  const int s = slab % a.Nss;
  const int col = tid % C;
  const int j = tid / C;
  const int n1 = tile * C + col;

  using W = typename SampleWord<FMT, NV>::type;
  const W* src = reinterpret_cast<const W*>(a.in) + (long long)c * a.chan_stride + (long long)s * (N1 * (long long)N2) + n1 +
                 (long long)N1 * j;
  float2 v[NV][R];
  {
    W w[R];
#pragma unroll
    for (int m = 0; m < R; ++m) w[m] = __ldg(src + (long long)N1 * T * m);
#pragma unroll
    for (int m = 0; m < R; ++m) {
      float2 smp[NV];
      unpack_word(w[m], smp);
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q][m] = smp[q];
    }
  }
  GroupFFT<N2, R, NV>::run(v, j, xch + (size_t)col * NV * smem_padded_len(N2), smem_padded_len(N2), tw_s,
                            BlockSyncL{});

  // Twiddle W_N^(n1*k2) and store.
  const int lomask = nlo - 1;
  float2* dst = a.scratch + (size_t)slab * NV * N2 * N1 + n1;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int k2 = j + m * T;
    const int e = n1 * k2;
    const float2 w = cmul(lo_s[e & lomask], hi_s[e >> a.h]);
#pragma unroll
    for (int q = 0; q < NV; ++q) dst[((size_t)q * N2 + k2) * N1] = cmul(v[q][m], w);
  }
}

template <int N1, int NV, int POL>
__global__ void __launch_bounds__(LargeCfg<N1>::TPB)
k_large_b(LargeLaunch a) {
  using Cf = LargeCfg<N1>;
  constexpr int R = Cf::R, T = Cf::T, C = Cf::C, TPB = Cf::TPB;
  constexpr int NP = PolOut<POL>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* xch = tw_s + N1;

  const int tid = threadIdx.x;
  for (int i = tid; i < N1; i += TPB) tw_s[i] = a.twN1[i];
  __syncthreads();

  const int N2 = 1 << a.logN2;
  const int N = N1 * N2;
  const int tiles = N2 / C;
  const int tile = blockIdx.x % tiles;
  const int uc = blockIdx.x / tiles;
  const int unit = uc / a.chunks;
  const int chunk = uc % a.chunks;
  const int c = unit / a.units_per_chan;
  const int d = unit % a.units_per_chan;
  const int row = tid % C;
  const int j = tid / C;
  const int k2 = tile * C + row;
  const int s_begin = chunk * a.spc;
  const int s_end = min(a.M, s_begin + a.spc);
  const float im_sign = a.conj ? -1.0f : 1.0f;

  float acc[R][NP];
#pragma unroll
  for (int m = 0; m < R; ++m)
#pragma unroll
    for (int p = 0; p < NP; ++p) acc[m][p] = 0.0f;

  float2* my_xch = xch + (size_t)row * NV * smem_padded_len(N1);
  for (int sl = s_begin; sl < s_end; ++sl) {
    const int slab = c * a.Nss + d * a.M + sl;
    const float2* src = a.scratch + ((size_t)slab * NV * N2 + k2) * N1 + j;
    float2 v[NV][R];
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
      for (int m = 0; m < R; ++m) v[q][m] = src[(size_t)q * N2 * N1 + m * T];
    GroupFFT<N1, R, NV>::run(v, j, my_xch, smem_padded_len(N1), tw_s, BlockSyncL{});
#pragma unroll
    for (int m = 0; m < R; ++m) {
      float2 x[NV];
#pragma unroll
      for (int q = 0; q < NV; ++q) x[q] = v[q][m];
      detect_acc<POL, NV>(acc[m], x, im_sign);
    }
  }

#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int f = k2 + N2 * (j + m * T);
#pragma unroll
    for (int p = 0; p < NP; ++p) {
      if (a.chunks > 1) {
        a.partial[(((size_t)unit * a.chunks + chunk) * NP + p) * N + f] = acc[m][p];
      } else {
        float* dst = a.out + (((size_t)d * NP + p) * a.Nc + c) * N + out_pos(f, N, a.inverse);
        if (a.mode == ACC_ADD) *dst += acc[m][p]; else *dst = acc[m][p];
      }
    }
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

template <int N2, int FMT, int NV>
cudaError_t launch_a_t(const LargeLaunch& L, cudaStream_t s, bool prep) {
  using Cf = LargeCfg<N2>;
  auto k = k_large_a<N2, FMT, NV>;
  const size_t smem = passA_smem<N2, NV>(L.h, L.logN);
  if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int N1 = 1 << L.logN1;
  const long long grid = (long long)(N1 / Cf::C) * L.Nc * L.Nss;
  k<<<(unsigned)grid, Cf::TPB, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N1, int NV, int POL>
cudaError_t launch_b_t(const LargeLaunch& L, cudaStream_t s, bool prep) {
  using Cf = LargeCfg<N1>;
  auto k = k_large_b<N1, NV, POL>;
  const size_t smem = passB_smem<N1, NV>();
  if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int N2 = 1 << L.logN2;
  const long long grid = (long long)(N2 / Cf::C) * L.n_units * L.chunks;
  k<<<(unsigned)grid, Cf::TPB, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N2>
cudaError_t launch_a_n(const LargeLaunch& L, cudaStream_t s, bool prep) {
  if (L.fmt == FMT_I16) return L.nv == 1 ? launch_a_t<N2, FMT_I16, 1>(L, s, prep) : launch_a_t<N2, FMT_I16, 2>(L, s, prep);
  return L.nv == 1 ? launch_a_t<N2, FMT_I8, 1>(L, s, prep) : launch_a_t<N2, FMT_I8, 2>(L, s, prep);
}

template <int N1>
cudaError_t launch_b_n(const LargeLaunch& L, cudaStream_t s, bool prep) {
  if (L.nv == 1) return launch_b_t<N1, 1, POL_TP>(L, s, prep);
  switch (L.pol) {
    case POL_FULL: return launch_b_t<N1, 2, POL_FULL>(L, s, prep);
    case POL_STOKES: return launch_b_t<N1, 2, POL_STOKES>(L, s, prep);
    default: return launch_b_t<N1, 2, POL_TP>(L, s, prep);
  }
}

cudaError_t dispatch_a(const LargeLaunch& L, cudaStream_t s, bool prep) {
  switch (L.logN2) {
    case 6: return launch_a_n<64>(L, s, prep);
    case 7: return launch_a_n<128>(L, s, prep);
    case 8: return launch_a_n<256>(L, s, prep);
    case 9: return launch_a_n<512>(L, s, prep);
    case 10: return launch_a_n<1024>(L, s, prep);
    case 11: return launch_a_n<2048>(L, s, prep);
    case 12: return launch_a_n<4096>(L, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

cudaError_t dispatch_b(const LargeLaunch& L, cudaStream_t s, bool prep) {
  switch (L.logN1) {
    case 6: return launch_b_n<64>(L, s, prep);
    case 7: return launch_b_n<128>(L, s, prep);
    case 8: return launch_b_n<256>(L, s, prep);
    case 9: return launch_b_n<512>(L, s, prep);
    case 10: return launch_b_n<1024>(L, s, prep);
    case 11: return launch_b_n<2048>(L, s, prep);
    case 12: return launch_b_n<4096>(L, s, prep);
    default: return cudaErrorInvalidValue;
  }
}

}  // namespace

int large_configure(LargeLaunch& L, int target_ctas, size_t* scratch_float2, size_t* partial_floats) {
  if (L.logN < 13 || L.logN > 24) return -1;
  L.logN2 = (L.logN + 1) / 2;
  L.logN1 = L.logN - L.logN2;
  L.h = (L.logN + 1) / 2;
  const int N1 = 1 << L.logN1, N2 = 1 << L.logN2;
  (void)N1;
  const int np = L.pol == POL_TP ? 1 : 4;
  // Chunks of a unit's spectra across CTAs for parallelism.
  int cpr;  // CTAs per unit and chunk
  switch (L.logN1) {
    case 6: cpr = N2 / LargeCfg<64>::C; break;
    case 7: cpr = N2 / LargeCfg<128>::C; break;
    case 8: cpr = N2 / LargeCfg<256>::C; break;
    case 9: cpr = N2 / LargeCfg<512>::C; break;
    case 10: cpr = N2 / LargeCfg<1024>::C; break;
    case 11: cpr = N2 / LargeCfg<2048>::C; break;
    default: cpr = N2 / LargeCfg<4096>::C; break;
  }
  const long long base = (long long)cpr * L.n_units;
  int chunks = (int)std::max<long long>(1, (target_ctas + base - 1) / base);
  chunks = std::min(chunks, L.M);
  L.spc = (L.M + chunks - 1) / chunks;
  L.chunks = (L.M + L.spc - 1) / L.spc;
  *scratch_float2 = (size_t)L.Nc * L.Nss * L.nv * ((size_t)1 << L.logN);
  *partial_floats = L.chunks > 1 ? (size_t)L.n_units * L.chunks * np * ((size_t)1 << L.logN) : 0;
  return 0;
}

cudaError_t large_prepare(const LargeLaunch& L) {
  cudaError_t e = dispatch_a(L, nullptr, true);
  if (e != cudaSuccess) return e;
  return dispatch_b(L, nullptr, true);
}

cudaError_t large_launch_a(const LargeLaunch& L, cudaStream_t s) { return dispatch_a(L, s, false); }
cudaError_t large_launch_b(const LargeLaunch& L, cudaStream_t s) { return dispatch_b(L, s, false); }

}  // namespace rsg
