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
//           spectra in registers, SNORM scale and the FFT-shifted store (or
//           add).
//
// X[k2 + N2 k1] = sum_n1 W_N1^(n1 k1) W_N^(n1 k2) sum_n2 x[n1 + N1 n2] W_N2^(n2 k2).
#include <algorithm>

#include "detect.cuh"
#include "fft_core.cuh"
#include "internal.h"

namespace rsg {

namespace {

constexpr int kRA = 16;  // radix of pass A
constexpr int kLargeTPB = 256;
// Resident CTAs per SM the register budget allows: one polarisation fits
// 80 registers a thread without spills (three CTAs of 256 threads), two
// polarisations need about 128 (two CTAs).
template <int NV>
constexpr int large_min_blocks() { return NV == 1 ? 3 : 2; }

// Sub-FFT of NSUB points at radix R; C sub-FFTs (columns or rows) per CTA,
// interleaved across lanes so that global accesses of neighbouring lanes are
// neighbouring columns.
template <int NSUB, int R>
struct LargeCfg {
  static constexpr int T = NSUB / R;              // threads per sub-FFT
  static constexpr int C = kLargeTPB / T > 8 ? 8 : (kLargeTPB / T > 0 ? kLargeTPB / T : 1);
  static constexpr int TPB = T * C;
  static constexpr int TW = stockham_tw_size(NSUB, R);
};

template <int POL>
__host__ __device__ constexpr int pass_b_radix() { return POL == POL_TP ? 16 : 8; }

struct BlockSyncL {
  __device__ __forceinline__ void operator()() const { __syncthreads(); }
};

// float2 between the exchange areas of neighbouring sub-FFTs (NV buffers of
// smem_padded_len(N) each): at least their size, and chosen so that the C
// sub-FFTs served by one half-warp start in different banks (their start
// offsets modulo 16 float2 are multiples of 16 / C), even for 16-byte rows.
template <int N, int C, int NV>
__host__ __device__ constexpr int sub_stride() {
  int base = NV * smem_padded_len(N);
  const int cp = C < 16 ? C : 16;
  const int want = (16 / cp) % 16;
  while (base % 16 != want) ++base;
  return base + (base & 1);
}

template <int N2, int NV>
constexpr size_t passA_smem() {
  using Cf = LargeCfg<N2, kRA>;
  return (size_t)((Cf::TW + 1) & ~1) * sizeof(float2) + (size_t)Cf::C * sub_stride<N2, Cf::C, NV>() * sizeof(float2);
}

template <int N1, int NV, int R>
constexpr size_t passB_smem() {
  using Cf = LargeCfg<N1, R>;
  return (size_t)((Cf::TW + 1) & ~1) * sizeof(float2) + (size_t)Cf::C * sub_stride<N1, Cf::C, NV>() * sizeof(float2);
}

}  // namespace

template <int N2, int FMT, int NV>
__global__ void __launch_bounds__(LargeCfg<N2, kRA>::TPB, large_min_blocks<NV>())
k_large_a(LargeLaunch a) {
  using Cf = LargeCfg<N2, kRA>;
  constexpr int R = kRA, T = Cf::T, C = Cf::C, TPB = Cf::TPB;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* xch = tw_s + ((Cf::TW + 1) & ~1);

  const int tid = threadIdx.x;
  for (int i = tid; i < Cf::TW; i += TPB) tw_s[i] = a.twN2[i];

  const int N1 = 1 << a.logN1;
  const int tiles = N1 / C;
  const int tile = blockIdx.x % tiles;
  const int slab = a.slab0 + blockIdx.x / tiles;
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
      Unpack<FMT, NV>::run(w[m], smp);
#pragma unroll
      for (int q = 0; q < NV; ++q) v[q][m] = smp[q];
    }
  }
  // W_N^(n1*j) for this thread's column, from the two-level table.
  const int e0 = n1 * j;
  const float2 w0 = cmul(__ldg(a.twLo + (e0 & ((1 << a.h) - 1))), __ldg(a.twHi + (e0 >> a.h)));
  __syncthreads();  // twiddle table in shared memory
  GroupFFT<N2, R, NV>::run(v, j, xch + (size_t)col * sub_stride<N2, C, NV>(), smem_padded_len(N2), tw_s,
                            BlockSyncL{});

  // Output k2 = j + m*T: W_N^(n1*k2) = W_N^(n1*j) * W_N^(n1*m*T).
  float2* dst = a.scratch + (size_t)slab * NV * N2 * N1 + n1;
  const float2* twm = a.twM + n1;
#pragma unroll
  for (int m = 0; m < R; ++m) {
    const int k2 = j + m * T;
    const float2 w = m == 0 ? w0 : cmul(w0, __ldg(twm + (size_t)m * N1));
#pragma unroll
    for (int q = 0; q < NV; ++q) dst[((size_t)q * N2 + k2) * N1] = cmul(v[q][m], w);
  }
}

template <int N1, int NV, int POL>
__global__ void __launch_bounds__(LargeCfg<N1, pass_b_radix<POL>()>::TPB, large_min_blocks<NV>())
k_large_b(LargeLaunch a) {
  constexpr int R = pass_b_radix<POL>();
  using Cf = LargeCfg<N1, R>;
  constexpr int T = Cf::T, C = Cf::C, TPB = Cf::TPB;
  constexpr int NP = PolOut<POL>::NP;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  float2* tw_s = reinterpret_cast<float2*>(smem_raw);
  float2* xch = tw_s + ((Cf::TW + 1) & ~1);

  const int tid = threadIdx.x;
  for (int i = tid; i < Cf::TW; i += TPB) tw_s[i] = a.twN1[i];
  __syncthreads();

  const int N2 = 1 << a.logN2;
  const int N = N1 * N2;
  const int tiles = N2 / C;
  const int tile = blockIdx.x % tiles;
  const int uc = blockIdx.x / tiles;
  const int unit = a.unit0 + uc / a.chunks;
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

  float2* my_xch = xch + (size_t)row * sub_stride<N1, C, NV>();
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

  if (a.chunks > 1) {
#pragma unroll
    for (int m = 0; m < R; ++m)
#pragma unroll
      for (int p = 0; p < NP; ++p)
        a.partial[(((size_t)unit * a.chunks + chunk) * NP + p) * N + k2 + N2 * (j + m * T)] = acc[m][p];
    return;
  }
  float* obase = a.out + ((size_t)d * NP * a.Nc + c) * N;
  const size_t plane = (size_t)a.Nc * N;
  if (a.mode == ACC_ADD) {
    // request every old value before the first store
    float old[R][NP];
#pragma unroll
    for (int m = 0; m < R; ++m)
#pragma unroll
      for (int p = 0; p < NP; ++p) old[m][p] = __ldcg(obase + p * plane + out_pos(k2 + N2 * (j + m * T), N, a.inverse));
#pragma unroll
    for (int m = 0; m < R; ++m)
#pragma unroll
      for (int p = 0; p < NP; ++p)
        obase[p * plane + out_pos(k2 + N2 * (j + m * T), N, a.inverse)] = __fmaf_rn(acc[m][p], a.scale, old[m][p]);
  } else {
#pragma unroll
    for (int m = 0; m < R; ++m)
#pragma unroll
      for (int p = 0; p < NP; ++p) obase[p * plane + out_pos(k2 + N2 * (j + m * T), N, a.inverse)] = acc[m][p] * a.scale;
  }
}

// ---------------------------------------------------------------------------
// Host side.
// ---------------------------------------------------------------------------
namespace {

template <int N2, int FMT, int NV>
cudaError_t launch_a_t(const LargeLaunch& L, cudaStream_t s, bool prep) {
  using Cf = LargeCfg<N2, kRA>;
  auto k = k_large_a<N2, FMT, NV>;
  const size_t smem = passA_smem<N2, NV>();
  if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int N1 = 1 << L.logN1;
  const long long grid = (long long)(N1 / Cf::C) * L.S;
  if (grid < 1) return cudaSuccess;
  k<<<(unsigned)grid, Cf::TPB, smem, s>>>(L);
  return cudaGetLastError();
}

template <int N1, int NV, int POL>
cudaError_t launch_b_t(const LargeLaunch& L, cudaStream_t s, bool prep) {
  constexpr int R = pass_b_radix<POL>();
  using Cf = LargeCfg<N1, R>;
  auto k = k_large_b<N1, NV, POL>;
  const size_t smem = passB_smem<N1, NV, R>();
  if (prep) return cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
  const int N2 = 1 << L.logN2;
  const long long grid = (long long)(N2 / Cf::C) * L.unit_count * L.chunks;
  if (grid < 1) return cudaSuccess;
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

template <int N1, int R>
int rows_per_cta() { return LargeCfg<N1, R>::C; }

int pass_b_rows(int logN1, int pol) {
  const bool tp = pol == POL_TP;
  switch (logN1) {
    case 6: return tp ? rows_per_cta<64, 16>() : rows_per_cta<64, 8>();
    case 7: return tp ? rows_per_cta<128, 16>() : rows_per_cta<128, 8>();
    case 8: return tp ? rows_per_cta<256, 16>() : rows_per_cta<256, 8>();
    case 9: return tp ? rows_per_cta<512, 16>() : rows_per_cta<512, 8>();
    case 10: return tp ? rows_per_cta<1024, 16>() : rows_per_cta<1024, 8>();
    case 11: return tp ? rows_per_cta<2048, 16>() : rows_per_cta<2048, 8>();
    default: return tp ? rows_per_cta<4096, 16>() : rows_per_cta<4096, 8>();
  }
}

}  // namespace

int large_pass_a_radix() { return kRA; }
int large_pass_b_radix(int pol) { return pol == POL_TP ? pass_b_radix<POL_TP>() : pass_b_radix<POL_FULL>(); }
int stockham_table_size(int N, int R) { return stockham_tw_size(N, R); }

int large_configure(LargeLaunch& L, int target_ctas, size_t* scratch_float2, size_t* partial_floats) {
  if (L.logN < 13 || L.logN > 24) return -1;
  L.logN2 = (L.logN + 1) / 2;
  L.logN1 = L.logN - L.logN2;
  L.h = (L.logN + 1) / 2;
  const int N2 = 1 << L.logN2;
  const int np = L.pol == POL_TP ? 1 : 4;
  // Chunks of a unit's spectra across CTAs for parallelism.
  const int cpr = N2 / pass_b_rows(L.logN1, L.pol);  // CTAs per unit and chunk
  const long long base = (long long)cpr * L.n_units;
  int chunks = (int)std::max<long long>(1, (target_ctas + base - 1) / base);
  chunks = std::min(chunks, L.M);
  L.spc = (L.M + chunks - 1) / chunks;
  L.chunks = (L.M + L.spc - 1) / L.spc;
  *scratch_float2 = (size_t)L.Nc * L.Nss * L.nv * ((size_t)1 << L.logN);
  *partial_floats = L.chunks > 1 ? (size_t)L.n_units * L.chunks * np * ((size_t)1 << L.logN) : 0;
  L.slab0 = 0;
  L.S = L.Nc * L.Nss;
  L.unit0 = 0;
  L.unit_count = L.n_units;
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
