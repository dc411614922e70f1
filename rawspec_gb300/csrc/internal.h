// internal.h -- launch descriptors shared by the host API (rawspec_api.cu)
// and the kernel translation units.  Plain C++ types only.
#pragma once

#include <cuda.h>
#include <cuda_runtime.h>

#include <cstddef>
#include <cstdint>

namespace rsg {

// Output polarisation modes (the reference's Npolout values, with total
// power split by the number of input polarisations).
enum PolMode : int { POL_TP = 0, POL_FULL = 4, POL_STOKES = -4 };

// Accumulation mode of a kernel's output.
enum AccMode : int { ACC_WRITE = 0, ACC_ADD = 1 };

// Sample formats of the device input buffer (int4 input is expanded to int8
// before processing).
enum SampleFormat : int { FMT_I8 = 0, FMT_I16 = 1 };

// ---------------------------------------------------------------------------
// Fused small-FFT product kernel (N <= 4096): unpack, FFT, detect, integrate.
// An "integration unit" is a run of M consecutive spectra of one channel that
// ends in one output spectrum (M = Na when an integration completes within
// the buffer, M = spectra per buffer otherwise).
// ---------------------------------------------------------------------------
struct SmallLaunch {
  // selection
  int logN = 0;      // log2 of the FFT length
  int fmt = 0;       // SampleFormat
  int nv = 2;        // input polarisations
  int pol = POL_TP;  // PolMode
  // geometry (filled by small_configure)
  int tpb = 0, sets = 1, chunks = 1, spc = 0, grid = 0;
  size_t smem = 0;
  // problem
  int Nc = 0, M = 0, units_per_chan = 0, n_units = 0;
  long long chan_stride = 0;  // samples per channel in the device buffer
  // buffers
  const void* in = nullptr;
  float* out = nullptr;       // [units_per_chan][|P|][Nc][N], FFT-shifted
  float* partial = nullptr;   // [n_units][chunks][|P|][N] (chunks > 1)
  const float2* tw = nullptr; // W_N^m, m < N
  // per call
  int mode = ACC_WRITE, inverse = 0, conj = 0;
  float scale = 1.0f;         // SNORM scale squared, applied to the results
  int vec16 = 0;              // spectra start on 16-byte boundaries (set by small_configure)
  int unit0 = 0, unit_count = 0;  // units of this launch (a channel range; all by default)
  // split of a unit for launches over a channel group (the pipelined path),
  // which see 1/pipe_groups of the units and need more CTAs per unit
  int chunks_pipe = 1, spc_pipe = 0;
};

// Chooses block size, units per block and chunks per unit.  target_ctas is
// the number of CTAs that fills the GPU.  Returns 0, or -1 if N is out of
// range.  partial_floats receives the scratch the launch needs (0 if none).
int small_configure(SmallLaunch& L, int target_ctas, size_t* partial_floats, int pipe_groups = 1);
cudaError_t small_launch(const SmallLaunch& L, cudaStream_t s);
// Up to kSmallGroupMax launches of the same kernel configuration (FFT length,
// sample format, polarisations, mode) in one grid, e.g. the buffers of
// several contexts: the entries keep their own buffers, units and splits.
constexpr int kSmallGroupMax = 8;
struct SmallGroup {
  SmallLaunch e[kSmallGroupMax];
  int end[kSmallGroupMax];  // prefix sums of the entries' grids
  int n = 0;
};
bool small_same_kernel(const SmallLaunch& a, const SmallLaunch& b);
cudaError_t small_launch_group(const SmallLaunch* L, int n, cudaStream_t s);
// Raises the kernel's dynamic shared-memory limit on the current device.
cudaError_t small_prepare(const SmallLaunch& L);

// Sums the per-chunk partial spectra of every unit in chunk order and writes
// (or adds) them FFT-shifted into the output.
struct FinalizeLaunch {
  const float* partial = nullptr;
  float* out = nullptr;
  int n_units = 0, chunks = 0, np = 1, N = 0, Nc = 0, units_per_chan = 0;
  int mode = ACC_WRITE, inverse = 0;
  float scale = 1.0f;
  int unit0 = 0;              // first unit; n_units counts the units of this launch
};
cudaError_t finalize_launch(const FinalizeLaunch& L, cudaStream_t s);

// ---------------------------------------------------------------------------
// Tensor-core DFT product kernel (k_tc.cu): N = S * S with S = 16, 32, 64,
// 8-bit input of two polarisations, units of a multiple of 64 / S spectra.
// Units, chunks, partial sums and outputs as in SmallLaunch.
// ---------------------------------------------------------------------------
struct TcLaunch {
  int logN = 0, pol = POL_TP;
  int Nc = 0, M = 0, units_per_chan = 0, n_units = 0;
  long long chan_stride = 0;     // samples per channel in the device buffer
  const void* in = nullptr;
  float* out = nullptr;          // [units_per_chan][|P|][Nc][N], FFT-shifted
  float* partial = nullptr;      // [n_units][chunks][|P|][N] (chunks > 1)
  const void* tab = nullptr;     // tc_table_bytes(logN) bytes from tc_table_fill
  int* err = nullptr;            // set to 1 if a bounded wait for the tensor cores timed out
  int mode = ACC_WRITE, inverse = 0, conj = 0;
  float scale = 1.0f;
  int unit0 = 0, unit_count = 0;
  int chunks = 1, spc = 0;       // chunks per unit, spectra per chunk (whole buffer)
  int chunks_pipe = 1, spc_pipe = 0;  // the same for a launch over one channel group
  int slots = 0;                 // resident CTAs on the device (the grid size cap)
  size_t smem = 0;
};
bool tc_supported(int logN, int fmt, int nv, int pol, int M);
size_t tc_table_bytes(int logN);
cudaError_t tc_table_fill(void* dst, int logN, cudaStream_t s);
// Sets the dynamic shared-memory limit, the grid cap and the chunking;
// partial_floats receives the scratch the launches need.  0, or -1.
int tc_configure(TcLaunch& L, size_t* partial_floats, int pipe_groups);
cudaError_t tc_launch(const TcLaunch& L, cudaStream_t s);
// The one-stage tensor-core kernel for N = 8, 16, 32 (k_tcs.cu), reached
// through the functions above.
bool tcs_supported(int logN, int fmt, int nv, int pol, int M);
size_t tcs_table_bytes(int logN);
cudaError_t tcs_table_fill(void* dst, int logN, cudaStream_t s);
cudaError_t tcs_plan(const TcLaunch& L, int* occ, size_t* smem);  // resident CTAs per SM, padded shared memory
cudaError_t tcs_launch(const TcLaunch& L, cudaStream_t s);

// ---------------------------------------------------------------------------
// Four-step large FFT (4096 < N <= 2^22): N = N1 * N2.
//   pass A: N2-point FFTs down the columns n1 of x[n1 + N1*n2], twiddled by
//           W_N^(n1*k2), written to scratch as [slab][pol][k2][n1];
//   pass B: N1-point FFTs along the rows k2, detection, integration.
// A slab is one (channel, spectrum) pair.
// ---------------------------------------------------------------------------
struct LargeLaunch {
  int logN = 0, logN1 = 0, logN2 = 0;
  int fmt = 0, nv = 2, pol = POL_TP;
  int Nc = 0, Nss = 0;            // channels, spectra per channel in a buffer
  int M = 0, units_per_chan = 0, n_units = 0, chunks = 1, spc = 0;
  long long chan_stride = 0;
  const void* in = nullptr;
  float2* scratch = nullptr;      // [Nc*Nss][nv][N2][N1]
  float* out = nullptr;
  float* partial = nullptr;
  const float2* twN2 = nullptr;   // pass-ordered Stockham table of the N2-point FFT
  const float2* twN1 = nullptr;   // pass-ordered Stockham table of the N1-point FFT
  const float2* twLo = nullptr;   // W_N^i, i < 2^h
  const float2* twHi = nullptr;   // W_N^(i*2^h), i < N / 2^h
  const float2* twM = nullptr;    // [m][n1] = W_N^(n1*m*T2), m < R_A, the pass-A output twiddles
  int h = 0;
  int mode = ACC_WRITE, inverse = 0, conj = 0;
  float scale = 1.0f;
  // persistent fused kernel (one spectrum per integration unit)
  int S = 0;                      // slabs of this launch (Nc * Nss for a whole buffer)
  int slab0 = 0;                  // first slab of this launch
  int unit0 = 0, unit_count = 0;  // units of this launch (two-kernel path)
  int ring = 0;                   // intermediate slots
  int lag = 2;                    // row tiles of slab s follow the column tiles of slab s + lag
  int lag_pipe = 2;               // the lag of a launch over one channel group of the pipelined call
  int* ctl = nullptr;             // [0] error, [1] CTAs finished, [2] item counter, [3..3+S) A done, [3+S..3+2S) B done
  int fused_ctas = 0;             // persistent grid size
  // fused kernel: tensor maps of the input (rows of N1 words), of the
  // twiddle tables twJ and twM and of the dump buffer (rows of N2 floats)
  const float2* twJ = nullptr;    // [j][n1] = W_N^(n1*j), j < N2 / R_A
  CUtensorMap tmap_in, tmap_twj, tmap_twm, tmap_out;
};
int large_configure(LargeLaunch& L, int target_ctas, size_t* scratch_float2, size_t* partial_floats);
// Radix of pass A (values per thread of its N2-point FFT) and its threads per
// column FFT, which define the pass-A twiddle table twM ([R_A][N1]).
int large_pass_a_radix();
// Sizes (entries) of the pass-ordered twiddle tables.
int stockham_table_size(int N, int R);
int small_radix(int logN, int pol);
int large_pass_b_radix(int pol);
cudaError_t large_launch_a(const LargeLaunch& L, cudaStream_t s);
cudaError_t large_launch_b(const LargeLaunch& L, cudaStream_t s);
// Raises both kernels' dynamic shared-memory limits on the current device.
cudaError_t large_prepare(const LargeLaunch& L);
// Persistent fused variant (k_large_fused.cu): supported for 8-bit input of
// two polarisations, 2^16 <= N <= 2^22 and integration units of one
// spectrum.  large_fused_plan() sets the grid size, the lag and the number of
// intermediate slabs (ring); the launch needs ring * 2 * N float2 of scratch
// and large_fused_ctl_ints() control words (zeroed once before the first
// launch; each launch leaves them zeroed for the next, the error word apart).
bool large_fused_supported(const LargeLaunch& L);
cudaError_t large_fused_plan(LargeLaunch& L);
int large_fused_row_radix(int pol);  // radix of the row tiles (twiddle table of twN1)
int large_fused_col_radix();         // radix of the column tiles (tables twN2 and twM)
int large_fused_ctl_ints(const LargeLaunch& L);
int large_fused_twj_entries(const LargeLaunch& L);  // size of the twJ table
cudaError_t large_fused_prepare(LargeLaunch& L);
cudaError_t large_fused_launch(const LargeLaunch& L, cudaStream_t s);

// ---------------------------------------------------------------------------
// Auxiliary kernels.
// ---------------------------------------------------------------------------
// W_n^m = exp(-2 pi i m stride / n) for m < count, computed in FP64 with
// sincospi and rounded to float.
cudaError_t twiddle_fill(float2* dst, long long count, long long n, long long stride, cudaStream_t s);
// Pass-ordered Stockham table of an N-point GroupFFT of radix R.
cudaError_t stockham_twiddle_fill(float2* dst, int N, int R, cudaStream_t s);
// dst[m*N1 + n1] = W_N^((n1*m*T) mod N) for m < R, n1 < N1.
cudaError_t passa_twiddle_fill(float2* dst, int N1, int R, long long T, long long N, cudaStream_t s);

// 4-bit complex expansion: for each of num_blocks blocks and each channel,
// bytes of the packed staging buffer become (re, im) int8 pairs in the input
// buffer (high nibble real, low nibble imaginary, sign-extended).
struct Expand4Launch {
  const uint8_t* packed = nullptr;  // [Nc][Nb*blk_bytes_packed]
  int8_t* out = nullptr;            // [Nc][Nb*blk_bytes_packed*2]
  int Nc = 0, Nb = 0;
  int c0 = 0, nch = -1;             // channel range (nch < 0: all channels)
  long long blk_bytes_packed = 0;   // Ntpb * Np
  int dst_block = 0, num_blocks = 0;
};
cudaError_t expand4_launch(const Expand4Launch& L, cudaStream_t s);

// Weighted incoherent sum over antennas of FFT-shifted spectra:
// ics[d][p][c][f] = sum_a w[a] * pwr[d][p][a*Nca + c][f] (sequential in a).
struct IcsLaunch {
  const float* pwr = nullptr;
  float* ics = nullptr;
  const float* w = nullptr;
  int Nd = 0, np = 1, Nc = 0, Nant = 1, N = 0;
};
cudaError_t ics_launch(const IcsLaunch& L, cudaStream_t s);

// Compensated (Kahan) integration across buffers, elementwise over n floats:
// y = stage - comp; t = sum + y; comp = (t - sum) - y; sum = t.  Products
// whose integration spans many buffers write each later buffer into `stage`
// and fold it into the running sum with this step.
cudaError_t kahan_merge_launch(float* sum, float* comp, const float* stage, long long n, cudaStream_t s);

}  // namespace rsg
