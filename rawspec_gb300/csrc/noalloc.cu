// noalloc.cu -- an entry point that computes one output product of one
// device-resident input buffer without allocating any memory.
//
// Some callers cannot call cudaMalloc: a streaming pipeline thread that must
// not stall (cudaMalloc/cudaFree synchronise the device and so block every
// other stream of the process), or a host framework that owns all device
// memory through its own pool and budget.  This entry point takes the input
// and output as caller-provided device pointers and keeps its only scratch --
// the per-chunk partial sums of the fused small-FFT kernel and its twiddle
// table -- in the file-scope array below, which every GPU that loads the
// library holds until the process exits.
#include <cstdint>
#include <cstdio>
#include <mutex>

#include "internal.h"
#include "rawspec_gb300.h"

namespace {

constexpr size_t kPartialFloats = size_t(1) << 20;  // 4 MiB of partial sums
constexpr int kMaxNt = 4096;                        // twiddle table capacity
constexpr size_t kScratchFloats = kPartialFloats + 2 * (size_t)kMaxNt;
constexpr int kMaxDevices = 64;

}  // namespace

// The shared scratch: partial sums [0, kPartialFloats), twiddles after them.
static __device__ __align__(256) float g_noalloc_scratch[kScratchFloats];

namespace {

std::mutex g_mu;
float* g_scratch_ptr[kMaxDevices] = {nullptr};

// Device address of the scratch array on the current device, looked up once
// per device.  In host code the array's name is only a host-side stand-in.
// The address belongs to the device's primary context (the one the CUDA
// runtime uses); it is not looked up again after cudaDeviceReset.
float* scratch_for_current_device() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return nullptr;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch_ptr[dev]) {
    float* p = nullptr;
    const cudaError_t rc = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_noalloc_scratch);
    if (rc != cudaSuccess) {
      fprintf(stderr, "rawspec_gb300_product_noalloc: cudaGetSymbolAddress failed: %s\n", cudaGetErrorName(rc));
      return nullptr;
    }
    g_scratch_ptr[dev] = p;
  }
  return g_scratch_ptr[dev];
}

bool pow2(unsigned x) { return x && !(x & (x - 1)); }

}  // namespace

#pragma GCC visibility push(default)
extern "C" int rawspec_gb300_product_noalloc(const void* d_in, unsigned int Nc, unsigned int Np, unsigned int Nbps,
                                             unsigned long long samples_per_channel, unsigned int Nt,
                                             unsigned int Na, int Npolout, int fft_dir, int input_conjugated,
                                             float* d_out, void* stream) {
  using namespace rsg;
  if (!d_in || !d_out || Nc == 0 || (Np != 1 && Np != 2) || (Nbps != 8 && Nbps != 16) || Na == 0) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: invalid arguments\n");
    return 1;
  }
  if (Npolout != 1 && Npolout != 4 && Npolout != -4) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: Npolout must be 1, 4 or -4, not %d\n", Npolout);
    return 1;
  }
  if (Npolout != 1 && Np != 2) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: Npolout %d needs two polarisations\n", Npolout);
    return 1;
  }
  // The kernels read one time sample (all polarisations) as one word.
  const unsigned word_bytes = Np * 2u * (Nbps / 8u);
  if ((reinterpret_cast<uintptr_t>(d_in) % word_bytes) != 0 || (reinterpret_cast<uintptr_t>(d_out) % 4) != 0) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: d_in must be aligned to %u bytes and d_out to 4 bytes\n",
            word_bytes);
    return 1;
  }
  if (!pow2(Nt) || Nt > (unsigned)kMaxNt) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: Nt (%u) must be a power of two no larger than %d\n", Nt, kMaxNt);
    return 1;
  }
  const unsigned long long span = (unsigned long long)Nt * Na;
  if (samples_per_channel == 0 || samples_per_channel % span != 0 || samples_per_channel / Nt > 0x7fffffffULL) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: Nt * Na (%llu) must divide the %llu samples per channel\n", span,
            samples_per_channel);
    return 1;
  }
  // integration units (channel x dump) are counted in int by the kernels
  if ((unsigned long long)Nc * (samples_per_channel / span) > 0x7fffffffULL) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: too many integrations (%u channels x %llu)\n", Nc,
            samples_per_channel / span);
    return 1;
  }
  float* scratch = scratch_for_current_device();
  if (!scratch) return 1;
  float2* tw = reinterpret_cast<float2*>(scratch + kPartialFloats);
  cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);

  const int npol = Npolout;
  SmallLaunch L;
  L.logN = 0;
  while ((1u << L.logN) < Nt) ++L.logN;
  L.fmt = Nbps == 16 ? FMT_I16 : FMT_I8;
  L.nv = (int)Np;
  L.pol = npol == 1 ? POL_TP : npol;
  L.Nc = (int)Nc;
  L.M = (int)Na;
  L.units_per_chan = (int)(samples_per_channel / span);
  L.n_units = (int)Nc * L.units_per_chan;
  L.chan_stride = (long long)samples_per_channel;
  L.in = d_in;
  L.out = d_out;
  L.tw = tw;
  L.partial = scratch;
  L.mode = ACC_WRITE;
  L.inverse = fft_dir <= 0 ? 1 : 0;
  L.conj = input_conjugated ? 1 : 0;
  const float snorm_d = Nbps == 16 ? 32767.0f : 127.0f;
  L.scale = 1.0f / (snorm_d * snorm_d);

  int sms = 152;
  int dev = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  // Split units over CTAs only as far as the partial sums fit the scratch.
  size_t need = 0;
  for (int target = sms * 4;; target /= 2) {
    if (small_configure(L, target, &need) != 0) {
      fprintf(stderr, "rawspec_gb300_product_noalloc: unsupported configuration\n");
      return 1;
    }
    if (need <= kPartialFloats || target <= 1) break;
  }
  if (need > kPartialFloats) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: partial sums exceed the %zu-float scratch\n", kPartialFloats);
    return 1;
  }
  cudaError_t e = stockham_twiddle_fill(tw, (int)Nt, small_radix(L.logN, L.pol), s);
  if (e == cudaSuccess) e = small_prepare(L);
  if (e == cudaSuccess) e = small_launch(L, s);
  if (e == cudaSuccess && L.chunks > 1) {
    FinalizeLaunch F;
    F.partial = scratch;
    F.out = d_out;
    F.n_units = L.n_units;
    F.chunks = L.chunks;
    F.np = npol == 1 ? 1 : 4;
    F.N = (int)Nt;
    F.Nc = (int)Nc;
    F.units_per_chan = L.units_per_chan;
    F.mode = ACC_WRITE;
    F.inverse = L.inverse;
    F.scale = L.scale;
    e = finalize_launch(F, s);
  }
  if (e != cudaSuccess) {
    fprintf(stderr, "rawspec_gb300_product_noalloc: %s\n", cudaGetErrorName(e));
    return 1;
  }
  return 0;
}
#pragma GCC visibility pop
