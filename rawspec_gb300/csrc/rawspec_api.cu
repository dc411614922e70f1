// rawspec_api.cu -- the C-ABI of the GB300-native librawspec.
//
// Implements the twelve entry points of rawspec.h (reference:
// rawspec_gpu.cu:404-1836) plus the extensions of rawspec_gb300.h.  The
// validation and normalisation rules of rawspec_initialize() follow the
// reference (rawspec_gpu.cu:471-641, 732-782) so that clients observe the same
// accepted configurations, coercions and error returns; the device-side
// design is this project's own:
//
//  * the device input buffer keeps the reference's corner-turned layout
//    [channel][Nb*Ntpb][pol][re,im] (one cudaMemcpy2DAsync per block);
//  * every product keeps one device accumulator laid out exactly like its
//    host dump buffer h_pwrbuf ([Nd][|P|][Nc][Nt], FFT-shifted), written by
//    the first buffer of an integration and added to by later ones, so a dump
//    is a single contiguous device->host copy and no clearing pass is needed;
//  * no channel batching: all Nc channels are processed by each launch, which
//    removes the batch cache kernels and their hazards;
//  * PRE_DUMP is queued before any write to h_pwrbuf/h_icsbuf of a dump and
//    POST_DUMP after both, on the processing stream (cudaLaunchHostFunc).
#include <algorithm>
#include <map>
#include <mutex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "internal.h"
#include "rawspec.h"
#include "rawspec_gb300.h"

#define RSG_STR1(s) #s
#define RSG_STR(s) RSG_STR1(s)
#ifndef RAWSPEC_GB300_VERSION
#define RAWSPEC_GB300_VERSION 0.1.0
#endif

namespace {

using namespace rsg;

constexpr int kMaxLogN = 24;
#ifndef RSG_COPY_GROUPS
#define RSG_COPY_GROUPS 8
#endif
constexpr int kMaxCopyGroups = RSG_COPY_GROUPS;       // channel groups of the pipelined copy
constexpr size_t kMinPipelinedBytes = size_t(16) << 20;  // smaller buffers are copied in one piece

#define RSG_CUDA(call)                                                                   \
  do {                                                                                   \
    cudaError_t rsg_e_ = (call);                                                         \
    if (rsg_e_ != cudaSuccess) {                                                         \
      fprintf(stderr, "got error %s at %s:%d\n", cudaGetErrorName(rsg_e_), __FILE__,     \
              __LINE__);                                                                 \
      fflush(stderr);                                                                    \
      return 1;                                                                          \
    }                                                                                    \
  } while (0)

struct Product {
  int N = 0, logN = 0, np = 1;
  unsigned Nss = 0, Nd = 0, Nis = 0, Na = 0;
  bool large = false;
  float* d_out = nullptr;
  size_t out_bytes = 0;
  float* d_ics = nullptr;
  size_t ics_bytes = 0;
  float2* d_tw = nullptr;  // small: Stockham table; large: A table | B table | lo | hi | pass-A output twiddles
  SmallLaunch sl;
  LargeLaunch ll;
  TcLaunch tl;
  int chunks = 1;
  bool fused = false;      // persistent fused four-step kernel
  bool tc = false;         // tensor-core DFT kernel instead of k_small
  int* d_ctl = nullptr;    // control words of the fused kernel (error word first) or the tc error word
  int* h_err = nullptr;    // pinned copy of the error word, refreshed after every fused or tc launch
  float* d_partial = nullptr;  // per-chunk partial sums of this product
  bool kahan = false;          // compensated integration across buffers
  float* d_stage = nullptr;    // this buffer's sums (out_bytes), folded into d_out by k_kahan_merge
  float* d_comp = nullptr;     // running compensation of d_out (out_bytes)
  CUtensorMap tmap_stage;      // the fused kernel's output map of d_stage
  float2* d_scratch = nullptr; // four-step intermediate (or the fused kernel's ring)
  cudaStream_t own_stream = nullptr;  // the product's kernels run concurrently with the others'
  cudaStream_t stream = nullptr;      // stream of the current buffer (own_stream, or the context
                                      // stream while profiling serialises the products)
  cudaEvent_t ev_join = nullptr;  // end of the product's work for a buffer
};

struct DumpCb {
  rawspec_context* ctx;
  int product;
};

struct EventPair {
  int cls;
  cudaEvent_t a, b;
};

struct GpuCtx {
  int device = 0;
  int sm_count = 152;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;     // host-to-device copies of the pipelined path
  cudaEvent_t ev_ready[kMaxCopyGroups] = {nullptr};  // per channel group: its copy has landed
  cudaEvent_t ev_free = nullptr;          // the previous buffer no longer needs the input
  cudaEvent_t ev_fork = nullptr;          // start of a buffer's work on the product streams
  void* d_in = nullptr;
  size_t in_bytes = 0;
  uint8_t* d_in4 = nullptr;
  size_t in4_bytes = 0;
  int fmt = FMT_I8;
  float* d_aws = nullptr;
  Product prod[MAX_OUTPUTS];
  unsigned inbuf_count = 0;
  int cur_mode[MAX_OUTPUTS] = {0};  // write / add of each product for the buffer being queued
  bool caller_managed = false;
  unsigned registered = 0;  // caller blocks examined (and page-locked unless they already were) so far
  std::vector<char> locked_here;  // per caller block: page-locked by this library (unlocked at cleanup)
  DumpCb cb[MAX_OUTPUTS];
  size_t device_bytes = 0;
  unsigned long long launches = 0;
  unsigned long long shared_launches = 0;  // launches that also carried other contexts' buffers
  // profiling
  bool profiling = false;
  std::vector<EventPair> pending;
  std::vector<cudaEvent_t> free_events;
  double prof_ms[RAWSPEC_GB300_K_COUNT] = {0};
  unsigned long long prof_n[RAWSPEC_GB300_K_COUNT] = {0};
  // rawspec_start_processing's work, captured once per pattern (each
  // product's write/add mode and dump, the direction, callbacks) and replayed
  struct Graph {
    cudaGraphExec_t exec;
    unsigned long long launches;
  };
  std::map<unsigned long long, Graph> graphs;
};

GpuCtx* G(rawspec_context* ctx) { return reinterpret_cast<GpuCtx*>(ctx->gpu_ctx); }

// ----------------------------------------------------------------------------
// Profiling helpers.
// ----------------------------------------------------------------------------
cudaEvent_t take_event(GpuCtx* g) {
  if (!g->free_events.empty()) {
    cudaEvent_t e = g->free_events.back();
    g->free_events.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
  return e;
}

struct ProfScope {
  GpuCtx* g;
  int cls;
  cudaStream_t st;
  cudaEvent_t a = nullptr;
  ProfScope(GpuCtx* g_, int cls_, cudaStream_t st_ = nullptr) : g(g_), cls(cls_), st(st_ ? st_ : g_->stream) {
    if (g->profiling) {
      a = take_event(g);
      if (a) cudaEventRecord(a, st);
    }
  }
  ~ProfScope() {
    if (g->profiling && a) {
      cudaEvent_t b = take_event(g);
      if (b) {
        cudaEventRecord(b, st);
        g->pending.push_back({cls, a, b});
      } else {
        g->free_events.push_back(a);
      }
    }
  }
};

void collect_profile(GpuCtx* g) {
  for (auto& p : g->pending) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
      g->prof_ms[p.cls] += ms;
      g->prof_n[p.cls] += 1;
    }
    g->free_events.push_back(p.a);
    g->free_events.push_back(p.b);
  }
  g->pending.clear();
}

// ----------------------------------------------------------------------------
// Validation (reference rules, rawspec_gpu.cu:471-641 and :732-760).
// ----------------------------------------------------------------------------
bool is_pow2(unsigned x) { return x && !(x & (x - 1)); }
int ilog2u(unsigned x) { int l = 0; while ((1u << l) < x) ++l; return l; }

// rawspec_start_processing replays CUDA graphs of its launches for input
// buffers below 128 MiB, where the host's launch calls are a measurable part
// of a buffer's time (the 4-antenna 4-bit Stokes shape, 64 MiB expanded:
// 0.243 against 0.250 ms per buffer); larger buffers launch directly (a graph
// of the production shape's three products measured 1-2 % slower: its
// branches start in another order).  RAWSPEC_GB300_GRAPHS=1 / =0 (read at
// each call) selects graphs always / never.
constexpr size_t kMaxGraphs = 64;
constexpr size_t kMaxGraphedBytes = size_t(128) << 20;
bool graphs_wanted(const GpuCtx* g) {
  const char* v = getenv("RAWSPEC_GB300_GRAPHS");
  if (v && v[0] == '0') return false;
  if (v && v[0] == '1') return true;
  return g->in_bytes < kMaxGraphedBytes;
}

// Which products of 8-bit input run their DFT on the tensor cores (k_tc)
// rather than in k_small: by default the total-power products of N = 1024,
// where k_tc is faster alone (227 against 233 us per 256 MiB buffer) and
// leaves FMA and issue slots to concurrent CUDA-core kernels.  Since k_small
// runs both polarisations on the packed f32x2 instructions it is the faster
// one at N = 4096 (299 against 339 us) and N = 256; the cross-pol modes stay
// on k_small (k_tc is as fast alone but slows a mixed step with the fused
// kernel).  RAWSPEC_GB300_TENSOR_DFT=1 at
// initialisation selects k_tc for every case it supports (N = 256, 1024,
// 4096, all modes up to 1024), =0 for none.  Without the variable, a
// tuning-table entry's dft= decides before the default.
bool tensor_dft_wanted(int logN, int pol, const rawspec_gb300_tune& t) {
  const char* v = getenv("RAWSPEC_GB300_TENSOR_DFT");
  if (v && v[0] == '0') return false;
  if (v && v[0] == '1') return true;
  if (t.dft >= 0) return t.dft == 1;
  return logN == 10 && pol == POL_TP;
}

// Tuning-table entry of product i of a validated context (unset values if
// the table has none).
rawspec_gb300_tune tune_for(const rawspec_context* ctx, int i) {
  rawspec_gb300_tune t;
  rawspec_gb300_tune_lookup(ctx->Nts[i], ctx->Nbps == 16 ? 16 : 8, ctx->Npolout[i], &t);
  return t;
}

// CTAs per SM the chunking of k_small and k_large_a/b aims for.
constexpr int kDefaultCtasPerSm = 4;
int target_ctas_for(int sm_count, const rawspec_gb300_tune& t) {
  return sm_count * (t.ctas > 0 ? t.ctas : kDefaultCtasPerSm);
}

// A tuning-table lag / ring of the fused kernel replaces the plan's; the
// ring stays longer than the lag, the lag of channel-group launches no
// longer than the ring allows.
void apply_fused_tune(LargeLaunch& L, const rawspec_gb300_tune& t) {
  const bool pipe_env = getenv("RAWSPEC_GB300_FUSED_LAG_PIPE") != nullptr;
  if (t.lag > 0) L.lag = t.lag;
  if (t.ring > 0) L.ring = t.ring;
  if (L.ring <= L.lag) L.ring = L.lag + 2;
  if (t.lag > 0 && !pipe_env) L.lag_pipe = L.lag;
  L.lag_pipe = std::max(1, std::min(L.lag_pipe, L.ring - 1));
}

// Products whose integration spans buffers (Nis > 1) and runs over at least
// 3072 spectra integrate across buffers with compensated (Kahan) summation:
// the first buffer of an integration writes the sum, every later one writes
// a staging plane that k_kahan_merge folds into the sum and its compensation
// plane.  Within a buffer the sums are already blocked (per-thread runs,
// chunk partials in fixed order), so the one long sequential chain is the
// chain across buffers.  RAWSPEC_GB300_KAHAN=1 / =0 at initialisation
// selects compensation for every product with Nis > 1 / for none.
constexpr unsigned kKahanMinNint = 3072;
bool kahan_wanted(unsigned Na, unsigned Nis) {
  if (Nis <= 1) return false;
  const char* v = getenv("RAWSPEC_GB300_KAHAN");
  if (v && v[0] == '0') return false;
  if (v && v[0] == '1') return true;
  return Na >= kKahanMinNint;
}

int validate_impl(rawspec_context* ctx, bool* expanded) {
  if (ctx->No == 0 || ctx->No > MAX_OUTPUTS) {
    fprintf(stderr, "output products must be in range [1..%d], not %d\n", MAX_OUTPUTS, ctx->No);
    fflush(stderr);
    return 1;
  }
  if (ctx->Np == 0 || ctx->Np > 2) {
    fprintf(stderr, "number of polarizations must be in range [1..2], not %d\n", ctx->Np);
    fflush(stderr);
    return 1;
  }
  for (unsigned i = 0; i < ctx->No; i++) {
    if (abs(ctx->Npolout[i]) != 4 || ctx->Np != 2) ctx->Npolout[i] = 1;
  }
  if (ctx->Ntpb == 0) {
    fprintf(stderr, "number of time samples per block cannot be zero\n");
    fflush(stderr);
    return 1;
  }
  if (ctx->Nbps == 0) ctx->Nbps = 8;
  if (ctx->Nbps != 4 && ctx->Nbps != 8 && ctx->Nbps != 16) {
    fprintf(stderr, "Number of bits per sample in raw header must be 4, 0/8, or 16\n");
    fprintf(stderr, "Observed a value of %d\n", ctx->Nbps);
    fflush(stderr);
    return 1;
  }
  *expanded = ctx->Nbps == 4;
  if (ctx->Nbps == 4) ctx->Nbps = 8;

  ctx->Ntmax = 0;
  for (unsigned i = 0; i < ctx->No; i++) {
    if (ctx->Nts[i] == 0) {
      fprintf(stderr, "Nts[%d] cannot be 0\n", i);
      fflush(stderr);
      return 1;
    }
    if (ctx->Ntmax < ctx->Nts[i]) ctx->Ntmax = ctx->Nts[i];
  }
  for (unsigned i = 0; i < ctx->No; i++) {
    if (ctx->Ntmax % ctx->Nts[i] != 0) {
      fprintf(stderr, "Nts[%d] (%u) is not a factor of Ntmax (%u)\n", i, ctx->Nts[i], ctx->Ntmax);
      fflush(stderr);
      return 1;
    }
  }
  if (ctx->Nb != 0) {
    if (((unsigned long long)ctx->Nb * ctx->Ntpb) % ctx->Ntmax != 0) {
      fprintf(stderr, "Ntmax (%u) is not a factor of Nb*Ntpb (%u * %u = %u)\n", ctx->Ntmax, ctx->Nb,
              ctx->Ntpb, ctx->Nb * ctx->Ntpb);
      fflush(stderr);
      return 1;
    }
  } else if (ctx->Ntmax < ctx->Ntpb) {
    if (ctx->Ntpb % ctx->Ntmax != 0) {
      fprintf(stderr, "Ntmax (%u) is not a factor of Ntpb (%u)\n", ctx->Ntmax, ctx->Ntpb);
      fflush(stderr);
      return 1;
    }
    ctx->Nb = 1;
  } else {
    if (ctx->Ntmax % ctx->Ntpb != 0) {
      fprintf(stderr, "Ntpb (%u) is not a factor of Nmax (%u)\n", ctx->Ntpb, ctx->Ntmax);
      fflush(stderr);
      return 1;
    }
    ctx->Nb = ctx->Ntmax / ctx->Ntpb;
  }
  if (ctx->Nb_host == 0 && ctx->h_blkbufs) {
    fprintf(stderr, "Must specify number of host input blocks when caller-managed\n");
    fflush(stderr);
    return 1;
  } else if (ctx->Nb_host == 0) {
    ctx->Nb_host = ctx->Nb;
  }
  const unsigned long long NbNtpb = (unsigned long long)ctx->Nb * ctx->Ntpb;
  for (unsigned i = 0; i < ctx->No; i++) {
    if (ctx->Nas[i] == 0) {
      fprintf(stderr, "Nas[%d] cannot be 0\n", i);
      fflush(stderr);
      return 1;
    }
    const unsigned long long ta = (unsigned long long)ctx->Nts[i] * ctx->Nas[i];
    if (ta < NbNtpb) {
      if (NbNtpb % ta != 0) {
        fprintf(stderr, "Nts[%d] * Nas[%d] (%u * %u) must divide Nb * Ntpb (%u * %u)\n", i, i, ctx->Nts[i],
                ctx->Nas[i], ctx->Nb, ctx->Ntpb);
        fflush(stderr);
        return 1;
      }
    } else if (ta % NbNtpb != 0) {
      fprintf(stderr, "Nb * Ntpb (%u * %u) must divide Nts[%d] * Nas[%d] (%u * %u)\n", ctx->Nb, ctx->Ntpb, i, i,
              ctx->Nts[i], ctx->Nas[i]);
      fflush(stderr);
      return 1;
    }
  }
  ctx->Nant = ctx->Nant == 0 ? 1 : ctx->Nant;
  if (ctx->Nbc == 0) {
    ctx->Nbc = ctx->Nc;
  } else {
    if (ctx->Nbc <= 1) {
      if (ctx->Nant > 1) {
        ctx->Nbc = ctx->Nc / ctx->Nant;
      } else {
        for (unsigned i = 1; i <= 10; i++)
          if (ctx->Nc % i == 0) ctx->Nbc = ctx->Nc / i;
      }
    }
    if (ctx->Nbc == 0 || ctx->Nc % ctx->Nbc != 0) {
      fprintf(stderr, "%d channels cannot be factorised to batches of %d\n", ctx->Nc, ctx->Nbc);
      return 1;
    }
    // Channel batching is accepted for compatibility; all channels are
    // processed together on the device.
  }

  // Limits of this implementation.
  if (ctx->Nc == 0) {
    fprintf(stderr, "number of coarse channels cannot be zero\n");
    fflush(stderr);
    return 1;
  }
  for (unsigned i = 0; i < ctx->No; i++) {
    if (!is_pow2(ctx->Nts[i]) || ilog2u(ctx->Nts[i]) > kMaxLogN) {
      fprintf(stderr, "Nts[%d] (%u) is not supported: FFT lengths must be powers of two up to 2^%d\n", i,
              ctx->Nts[i], kMaxLogN);
      fflush(stderr);
      return 1;
    }
  }
  if (ctx->incoherently_sum) {
    if (ctx->Nc % ctx->Nant != 0) {
      fprintf(stderr, "%d channels cannot be split among %d antennas\n", ctx->Nc, ctx->Nant);
      fflush(stderr);
      return 1;
    }
    if (!ctx->Aws || !((ctx->Naws == 1 && ctx->Naws < (int)ctx->Nant) || ctx->Naws == (int)ctx->Nant)) {
      fprintf(stderr, "Not enough antenna-weights provided for the %d antennas: only provided %d.\n", ctx->Nant,
              ctx->Naws);
      fflush(stderr);
      return 1;
    }
  }

  for (unsigned i = 0; i < ctx->No; i++) {
    const unsigned Nss = (unsigned)(NbNtpb / ctx->Nts[i]);
    ctx->Nds[i] = Nss / ctx->Nas[i];
    if (ctx->Nds[i] == 0) ctx->Nds[i] = 1;
    ctx->h_pwrbuf_size[i] = (size_t)abs(ctx->Npolout[i]) * ctx->Nds[i] * ctx->Nts[i] * ctx->Nc * sizeof(float);
  }
  return 0;
}

void derived(const rawspec_context* ctx, int i, unsigned* Nss, unsigned* Nis, unsigned* Nd) {
  const unsigned long long NbNtpb = (unsigned long long)ctx->Nb * ctx->Ntpb;
  *Nss = (unsigned)(NbNtpb / ctx->Nts[i]);
  *Nd = *Nss / ctx->Nas[i];
  if (*Nd == 0) *Nd = 1;
  *Nis = ctx->Nas[i] / *Nss;
  if (*Nis == 0) *Nis = 1;
}

// ----------------------------------------------------------------------------
// Host callbacks (run on a CUDA host-function thread; no CUDA calls).
// ----------------------------------------------------------------------------
void CUDART_CB pre_dump_fn(void* data) {
  DumpCb* d = reinterpret_cast<DumpCb*>(data);
  if (d->ctx->dump_callback) d->ctx->dump_callback(d->ctx, d->product, RAWSPEC_CALLBACK_PRE_DUMP);
}
void CUDART_CB post_dump_fn(void* data) {
  DumpCb* d = reinterpret_cast<DumpCb*>(data);
  if (d->ctx->dump_callback) d->ctx->dump_callback(d->ctx, d->product, RAWSPEC_CALLBACK_POST_DUMP);
}

// ----------------------------------------------------------------------------
// Memory.  Device buffers come from the device's stream-ordered memory pool
// (cudaMallocAsync on the context stream, freed with cudaFreeAsync), which
// keeps up to 8 GiB of freed memory for later contexts (the rest returns to
// the driver) and never synchronises the device, so that creating and freeing
// contexts does not stall other contexts' work (a job server runs many).
// Page-locked host buffers (h_pwrbuf, h_icsbuf, the library's host blocks)
// are likewise kept by size class for later contexts, up to 8 GiB: pinning
// memory costs milliseconds per allocation.
// ----------------------------------------------------------------------------
void keep_pool_memory(int device) {
  static std::mutex mu;
  static std::vector<int> done;
  std::lock_guard<std::mutex> g(mu);
  if (std::find(done.begin(), done.end(), device) != done.end()) return;
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = uint64_t(8) << 30;  // freed bytes the pool keeps (this process's memory only)
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  }
  cudaGetLastError();
  done.push_back(device);
}

std::mutex g_pin_mu;
std::multimap<size_t, void*> g_pin_cache;  // size class -> buffer
size_t g_pin_cached = 0;
constexpr size_t kPinCacheCap = size_t(8) << 30;

// Allocation size of a pinned request: a multiple of a quarter of the
// largest power of two not above it (at most 25 % more), 4 KiB at least.
size_t pin_class(size_t bytes) {
  if (bytes <= 4096) return 4096;
  size_t p = 1;
  while (p * 2 <= bytes) p *= 2;
  const size_t q = p / 4;
  return (bytes + q - 1) / q * q;
}

cudaError_t pinned_alloc(void** ptr, size_t bytes) {
  const size_t c = pin_class(bytes);
  {
    std::lock_guard<std::mutex> g(g_pin_mu);
    auto it = g_pin_cache.find(c);
    if (it != g_pin_cache.end()) {
      *ptr = it->second;
      g_pin_cache.erase(it);
      g_pin_cached -= c;
      return cudaSuccess;
    }
  }
  return cudaHostAlloc(ptr, c, cudaHostAllocDefault);
}

// The buffer must no longer be used by any stream.
void pinned_free(void* ptr, size_t bytes) {
  if (!ptr) return;
  const size_t c = pin_class(bytes);
  {
    std::lock_guard<std::mutex> g(g_pin_mu);
    if (g_pin_cached + c <= kPinCacheCap) {
      g_pin_cache.emplace(c, ptr);
      g_pin_cached += c;
      return;
    }
  }
  cudaFreeHost(ptr);
}

template <typename T>
int dev_alloc(GpuCtx* g, T** p, size_t bytes) {
  if (bytes == 0) {
    *p = nullptr;
    return 0;
  }
  void* v = nullptr;
  cudaError_t e = cudaMallocAsync(&v, bytes, g->stream);
  if (e != cudaSuccess) {
    fprintf(stderr, "got error %s allocating %zu bytes of device memory\n", cudaGetErrorName(e), bytes);
    fflush(stderr);
    return 1;
  }
  g->device_bytes += bytes;
  *p = reinterpret_cast<T*>(v);
  return 0;
}

int launch_finalize(rawspec_context* ctx, GpuCtx* g, const Product& P, float* out, int unit0, int n_units, int chunks,
                    int upc, int mode, int inverse, float scale) {
  FinalizeLaunch F;
  F.partial = P.d_partial;
  F.out = out;
  F.unit0 = unit0;
  F.n_units = n_units;
  F.chunks = chunks;
  F.np = P.np;
  F.N = P.N;
  F.Nc = (int)ctx->Nc;
  F.units_per_chan = upc;
  F.mode = mode;
  F.inverse = inverse;
  F.scale = scale;
  ProfScope ps(g, RAWSPEC_GB300_K_FINALIZE, P.stream);
  RSG_CUDA(finalize_launch(F, P.stream));
  g->launches++;
  return 0;
}

// A k_small launch held back so that it can share one grid with launches
// of other contexts (rawspec_gb300_start_processing_group).
struct DeferredSmall {
  rawspec_context* ctx;
  GpuCtx* g;
  int product;
  SmallLaunch L;
  float* out;
};

// Queues product i's kernels for the channels [c0, c1) of the buffer.  With
// compensated integration the buffers after an integration's first write
// their sums to the staging plane.  With `defer`, a k_small launch over all
// channels is recorded there instead (with its finalisation).
int launch_product(rawspec_context* ctx, GpuCtx* g, int i, int mode, int inverse, int c0, int c1,
                   std::vector<DeferredSmall>* defer = nullptr) {
  Product& P = g->prod[i];
  const bool staged = P.kahan && mode == ACC_ADD;
  float* const out = staged ? P.d_stage : P.d_out;
  if (staged) mode = ACC_WRITE;
  if (P.tc) {
    TcLaunch L = P.tl;
    L.out = out;
    L.mode = mode;
    L.inverse = inverse;
    L.unit0 = c0 * L.units_per_chan;
    L.unit_count = (c1 - c0) * L.units_per_chan;
    if (c1 - c0 < (int)ctx->Nc) {  // a channel group: the finer split
      L.chunks = L.chunks_pipe;
      L.spc = L.spc_pipe;
    }
    {
      ProfScope ps(g, RAWSPEC_GB300_K_TC, P.stream);
      RSG_CUDA(tc_launch(L, P.stream));
      g->launches++;
    }
    if (L.chunks > 1 &&
        launch_finalize(ctx, g, P, out, L.unit0, L.unit_count, L.chunks, L.units_per_chan, mode, inverse, L.scale))
      return 1;
    RSG_CUDA(cudaMemcpyAsync(P.h_err, P.d_ctl, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
    return 0;
  }
  if (!P.large) {
    SmallLaunch L = P.sl;
    L.out = out;
    L.mode = mode;
    L.inverse = inverse;
    L.unit0 = c0 * L.units_per_chan;
    L.unit_count = (c1 - c0) * L.units_per_chan;
    if (c1 - c0 < (int)ctx->Nc) {  // a channel group: the finer split
      L.chunks = L.chunks_pipe;
      L.spc = L.spc_pipe;
    } else if (defer && !g->profiling) {
      defer->push_back(DeferredSmall{ctx, g, i, L, out});
      return 0;
    }
    {
      ProfScope ps(g, RAWSPEC_GB300_K_SMALL, P.stream);
      RSG_CUDA(small_launch(L, P.stream));
      g->launches++;
    }
    if (L.chunks > 1 &&
        launch_finalize(ctx, g, P, out, L.unit0, L.unit_count, L.chunks, L.units_per_chan, mode, inverse, L.scale))
      return 1;
  } else {
    LargeLaunch L = P.ll;
    L.out = out;
    if (staged) L.tmap_out = P.tmap_stage;
    L.mode = mode;
    L.inverse = inverse;
    L.slab0 = c0 * L.Nss;
    L.S = (c1 - c0) * L.Nss;
    L.unit0 = c0 * L.units_per_chan;
    L.unit_count = (c1 - c0) * L.units_per_chan;
    if (c1 - c0 < (int)ctx->Nc) L.lag = L.lag_pipe;  // a channel group: its own lag
    if (P.fused) {
      {
        ProfScope ps(g, RAWSPEC_GB300_K_LARGE_FUSED, P.stream);
        RSG_CUDA(large_fused_launch(L, P.stream));
        g->launches++;
      }
      // the error word follows the launch to the host, so that a wait needs no
      // synchronous copy
      RSG_CUDA(cudaMemcpyAsync(P.h_err, P.d_ctl, sizeof(int), cudaMemcpyDeviceToHost, P.stream));
      return 0;
    }
    {
      ProfScope ps(g, RAWSPEC_GB300_K_LARGE_A, P.stream);
      RSG_CUDA(large_launch_a(L, P.stream));
      g->launches++;
    }
    {
      ProfScope ps(g, RAWSPEC_GB300_K_LARGE_B, P.stream);
      RSG_CUDA(large_launch_b(L, P.stream));
      g->launches++;
    }
    if (L.chunks > 1 &&
        launch_finalize(ctx, g, P, out, L.unit0, L.unit_count, L.chunks, L.units_per_chan, mode, inverse, L.scale))
      return 1;
  }
  return 0;
}

// Queues one input buffer's kernels: each product's, on the product's own
// stream, over `ngroups` channel groups (group k waits for ready[k] when
// given).  With `defer`, k_small launches over all channels are recorded
// there instead of queued (the caller queues them, then buffer_finish).
int buffer_launches(rawspec_context* ctx, GpuCtx* g, int fft_dir, int ngroups, const cudaEvent_t* ready,
                    std::vector<DeferredSmall>* defer) {
  const int inverse = fft_dir <= 0 ? 1 : 0;
  g->inbuf_count++;
  RSG_CUDA(cudaEventRecord(g->ev_fork, g->stream));
  for (unsigned i = 0; i < ctx->No; i++) {
    Product& P = g->prod[i];
    P.stream = g->profiling ? g->stream : P.own_stream;
    RSG_CUDA(cudaStreamWaitEvent(P.stream, g->ev_fork, 0));
  }
  int* mode = g->cur_mode;
  for (unsigned i = 0; i < ctx->No; i++)
    mode[i] = ((g->inbuf_count - 1) % g->prod[i].Nis == 0) ? ACC_WRITE : ACC_ADD;
  for (int grp = 0; grp < ngroups; grp++) {
    const int c0 = (int)((long long)grp * ctx->Nc / ngroups);
    const int c1 = (int)((long long)(grp + 1) * ctx->Nc / ngroups);
    if (c1 <= c0) continue;
    for (unsigned i = 0; i < ctx->No; i++) {
      if (ready) RSG_CUDA(cudaStreamWaitEvent(g->prod[i].stream, ready[grp], 0));
      if (launch_product(ctx, g, (int)i, mode[i], inverse, c0, c1, defer)) return 1;
    }
  }
  return 0;
}

// After a buffer's kernels: the compensated integration merge, and the dumps
// of the products whose integration completes, each on the product's
// stream; the context stream joins all of them.
int buffer_finish(rawspec_context* ctx, GpuCtx* g) {
  const int* mode = g->cur_mode;
  for (unsigned i = 0; i < ctx->No; i++) {
    Product& P = g->prod[i];
    if (P.kahan) {
      const long long n = (long long)(P.out_bytes / sizeof(float));
      if (mode[i] == ACC_WRITE) {
        RSG_CUDA(cudaMemsetAsync(P.d_comp, 0, P.out_bytes, P.stream));
      } else {
        ProfScope ps(g, RAWSPEC_GB300_K_MERGE, P.stream);
        RSG_CUDA(kahan_merge_launch(P.d_out, P.d_comp, P.d_stage, n, P.stream));
        g->launches++;
      }
    }
    if (g->inbuf_count % P.Nis == 0) {
      if (ctx->incoherently_sum) {
        IcsLaunch I;
        I.pwr = P.d_out;
        I.ics = P.d_ics;
        I.w = g->d_aws;
        I.Nd = (int)P.Nd;
        I.np = P.np;
        I.Nc = (int)ctx->Nc;
        I.Nant = (int)ctx->Nant;
        I.N = P.N;
        ProfScope ps(g, RAWSPEC_GB300_K_ICS, P.stream);
        RSG_CUDA(ics_launch(I, P.stream));
        g->launches++;
      }
      // Host functions are queued only when a callback is installed (a NULL
      // callback would be a no-op on the callback thread anyway).
      const bool cb = ctx->dump_callback != nullptr;
      if (cb) RSG_CUDA(cudaLaunchHostFunc(P.stream, pre_dump_fn, &g->cb[i]));
      {
        ProfScope ps(g, RAWSPEC_GB300_K_D2H, P.stream);
        RSG_CUDA(cudaMemcpyAsync(ctx->h_pwrbuf[i], P.d_out, P.out_bytes, cudaMemcpyDeviceToHost, P.stream));
        if (ctx->incoherently_sum)
          RSG_CUDA(cudaMemcpyAsync(ctx->h_icsbuf[i], P.d_ics, P.ics_bytes, cudaMemcpyDeviceToHost, P.stream));
      }
      if (cb) RSG_CUDA(cudaLaunchHostFunc(P.stream, post_dump_fn, &g->cb[i]));
    }
    RSG_CUDA(cudaEventRecord(P.ev_join, P.stream));
    RSG_CUDA(cudaStreamWaitEvent(g->stream, P.ev_join, 0));
  }
  return 0;
}


// Processes one input buffer (buffer_launches, then buffer_finish).
int process_buffer(rawspec_context* ctx, GpuCtx* g, int fft_dir, int ngroups, const cudaEvent_t* ready) {
  if (buffer_launches(ctx, g, fft_dir, ngroups, ready, nullptr)) return 1;
  return buffer_finish(ctx, g);
}

// Queues the deferred k_small launches of several contexts: launches of the
// same kernel configuration share one grid (up to kSmallGroupMax), issued on
// the first one's product stream after every member's stream has reached
// it; each member's stream then continues after the shared launch with its
// own finalisation.
int launch_deferred(std::vector<DeferredSmall>& d) {
  std::vector<char> done(d.size(), 0);
  for (size_t a = 0; a < d.size(); a++) {
    if (done[a]) continue;
    std::vector<size_t> mem{a};
    done[a] = 1;
    for (size_t b = a + 1; b < d.size() && (int)mem.size() < kSmallGroupMax; b++)
      if (!done[b] && small_same_kernel(d[a].L, d[b].L)) {
        mem.push_back(b);
        done[b] = 1;
      }
    Product& Pa = d[a].g->prod[d[a].product];
    cudaStream_t st = Pa.stream;
    std::vector<SmallLaunch> Ls;
    for (size_t m : mem) {
      Ls.push_back(d[m].L);
      if (m == a) continue;
      GpuCtx* gm = d[m].g;
      cudaEvent_t ev = take_event(gm);
      if (!ev) return 1;
      RSG_CUDA(cudaEventRecord(ev, gm->prod[d[m].product].stream));
      RSG_CUDA(cudaStreamWaitEvent(st, ev, 0));
      gm->free_events.push_back(ev);  // the wait has taken the event's state
    }
    if (mem.size() == 1) {
      RSG_CUDA(small_launch(Ls[0], st));
    } else {
      RSG_CUDA(small_launch_group(Ls.data(), (int)Ls.size(), st));
      cudaEvent_t done_ev = take_event(d[a].g);
      if (!done_ev) return 1;
      RSG_CUDA(cudaEventRecord(done_ev, st));
      for (size_t m : mem)
        if (m != a) RSG_CUDA(cudaStreamWaitEvent(d[m].g->prod[d[m].product].stream, done_ev, 0));
      d[a].g->free_events.push_back(done_ev);
    }
    for (size_t m : mem) {
      DeferredSmall& e = d[m];
      e.g->launches++;  // every member's context counts the launch it took part in
      if (mem.size() > 1) e.g->shared_launches++;
      Product& P = e.g->prod[e.product];
      if (e.L.chunks > 1 && launch_finalize(e.ctx, e.g, P, e.out, e.L.unit0, e.L.unit_count, e.L.chunks,
                                            e.L.units_per_chan, e.L.mode, e.L.inverse, e.L.scale))
        return 1;
    }
  }
  return 0;
}

}  // namespace

// Device bytes rawspec_initialize() allocates for a validated context: the
// same sizes, from the same configuration functions, without allocating.
int plan_device_bytes(const rawspec_context* ctx, bool expanded, int sm_count, size_t* total) {
  size_t t = 0;
  const int fmt = ctx->Nbps == 16 ? FMT_I16 : FMT_I8;
  const size_t blk_bytes = (size_t)ctx->Ntpb * ctx->Np * ctx->Nc * 2 * (ctx->Nbps / 8);
  const size_t in_bytes = blk_bytes * ctx->Nb;
  t += in_bytes;
  if (expanded) t += in_bytes / 2;
  if (ctx->incoherently_sum) t += ctx->Nant * sizeof(float);
  const int groups = std::min<int>(kMaxCopyGroups, (int)ctx->Nc);
  auto al = [](size_t n) { return (n + 31) & ~size_t(31); };
  for (unsigned i = 0; i < ctx->No; i++) {
    const int N = (int)ctx->Nts[i], logN = ilog2u(ctx->Nts[i]), np = abs(ctx->Npolout[i]);
    unsigned Nss, Nis, Nd;
    derived(ctx, (int)i, &Nss, &Nis, &Nd);
    const int pol = np == 1 ? POL_TP : ctx->Npolout[i];
    const int M = (int)(Nis > 1 ? Nss : ctx->Nas[i]);
    const int upc = (int)(Nis > 1 ? 1 : Nss / ctx->Nas[i]);
    const rawspec_gb300_tune tune = tune_for(ctx, (int)i);
    const int target_ctas = target_ctas_for(sm_count, tune);
    t += ctx->h_pwrbuf_size[i];
    if (kahan_wanted(ctx->Nas[i], Nis)) t += 2 * ctx->h_pwrbuf_size[i];
    if (ctx->incoherently_sum) t += ctx->h_pwrbuf_size[i] / ctx->Nant;
    const bool large = logN > 12;
    if (!large && tensor_dft_wanted(logN, pol, tune) && tc_supported(logN, fmt, (int)ctx->Np, pol, M)) {
      TcLaunch L;
      L.logN = logN;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      size_t pf = 0;
      if (tc_configure(L, &pf, groups)) return 1;
      t += pf * sizeof(float) + ((tc_table_bytes(logN) + 15) & ~size_t(15)) + sizeof(int);
    } else if (!large) {
      SmallLaunch L;
      L.logN = logN;
      L.fmt = fmt;
      L.nv = (int)ctx->Np;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      L.chan_stride = (long long)ctx->Nb * ctx->Ntpb;
      size_t pf = 0;
      if (small_configure(L, target_ctas, &pf, groups)) return 1;
      t += pf * sizeof(float) + (size_t)std::max(stockham_table_size(N, small_radix(logN, pol)), 1) * sizeof(float2);
    } else {
      LargeLaunch L;
      L.logN = logN;
      L.fmt = fmt;
      L.nv = (int)ctx->Np;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.Nss = (int)Nss;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      L.chan_stride = (long long)ctx->Nb * ctx->Ntpb;
      size_t sf = 0, pf = 0;
      if (large_configure(L, target_ctas, &sf, &pf)) return 1;
      const bool fused = large_fused_supported(L);
      if (fused) {
        L.S = (int)ctx->Nc * (int)Nss;
        if (large_fused_plan(L) != cudaSuccess) return 1;
        apply_fused_tune(L, tune);
        sf = (size_t)std::min(L.ring, L.S) * L.nv * ((size_t)1 << L.logN);
        pf = 0;
        t += (size_t)large_fused_ctl_ints(L) * sizeof(int);
      }
      t += sf * sizeof(float2) + pf * sizeof(float);
      const int n1 = 1 << L.logN1, n2 = 1 << L.logN2;
      const int RA = fused ? large_fused_col_radix() : large_pass_a_radix();
      const int RB = fused ? large_fused_row_radix(pol) : large_pass_b_radix(pol);
      const size_t ta = (size_t)stockham_table_size(n2, RA), tb = (size_t)stockham_table_size(n1, RB);
      const size_t nlo = (size_t)1 << L.h, nhi = (size_t)1 << (L.logN - L.h), nm = (size_t)RA * n1;
      const size_t nj = fused ? (size_t)large_fused_twj_entries(L) : 0;
      const size_t o_j = al(ta) + al(tb) + al(nlo) + al(nhi) + al(nm);
      t += (o_j + nj) * sizeof(float2);
    }
  }
  *total = t;
  return 0;
}

// ============================================================================
// Public C interface (the only symbols the library exports).
// ============================================================================
#pragma GCC visibility push(default)
extern "C" {

const char* get_librawspec_version() { return RSG_STR(RAWSPEC_GB300_VERSION) "-gb300"; }

const char* get_cufft_version() { return "none (native sm_103a FFT)"; }

int rawspec_gb300_product_kernel(rawspec_context* ctx, int product) {
  GpuCtx* g = G(ctx);
  if (!g || product < 0 || product >= (int)ctx->No) return -1;
  const Product& P = g->prod[product];
  if (P.tc) return RAWSPEC_GB300_K_TC;
  if (!P.large) return RAWSPEC_GB300_K_SMALL;
  return P.fused ? RAWSPEC_GB300_K_LARGE_FUSED : RAWSPEC_GB300_K_LARGE_A;
}

int rawspec_gb300_validate(rawspec_context* ctx) {
  bool expanded = false;
  return validate_impl(ctx, &expanded);
}

int rawspec_gb300_product_info(const rawspec_context* ctx, int product, unsigned* Nss, unsigned* Nis,
                               unsigned* Nd) {
  if (!ctx || product < 0 || product >= (int)ctx->No || ctx->Nb == 0 || ctx->Nts[product] == 0 ||
      ctx->Nas[product] == 0)
    return 1;
  unsigned a, b, c;
  derived(ctx, product, &a, &b, &c);
  if (Nss) *Nss = a;
  if (Nis) *Nis = b;
  if (Nd) *Nd = c;
  return 0;
}

int rawspec_initialize(rawspec_context* ctx) {
  bool expanded = false;
  if (validate_impl(ctx, &expanded)) return 1;
  if (ctx->Nbc != ctx->Nc)
    printf("Batching %d channels into %d batches of %d.\n", ctx->Nc, ctx->Nc / ctx->Nbc, ctx->Nbc);

  for (int i = 0; i < MAX_OUTPUTS; i++) {
    ctx->h_pwrbuf[i] = nullptr;
    ctx->h_icsbuf[i] = nullptr;
  }
  ctx->gpu_ctx = nullptr;

  cudaError_t rc = cudaSetDevice(ctx->gpu_index);
  if (rc != cudaSuccess) {
    fprintf(stderr, "got error %s at %s:%d\n", cudaGetErrorName(rc), __FILE__, __LINE__);
    fflush(stderr);
    return 1;
  }
  GpuCtx* g = new (std::nothrow) GpuCtx();
  if (!g) {
    fprintf(stderr, "unable to allocate rawspec GPU context\n");
    return 1;
  }
  ctx->gpu_ctx = g;
  g->device = ctx->gpu_index;
  cudaDeviceGetAttribute(&g->sm_count, cudaDevAttrMultiProcessorCount, g->device);
  for (int i = 0; i < MAX_OUTPUTS; i++) g->cb[i] = {ctx, i};
  g->fmt = ctx->Nbps == 16 ? FMT_I16 : FMT_I8;

#define FAIL()             \
  do {                     \
    rawspec_cleanup(ctx);  \
    return 1;              \
  } while (0)
#define CK(call)                                                                                   \
  do {                                                                                             \
    cudaError_t e_ = (call);                                                                       \
    if (e_ != cudaSuccess) {                                                                       \
      fprintf(stderr, "got error %s at %s:%d\n", cudaGetErrorName(e_), __FILE__, __LINE__);        \
      fflush(stderr);                                                                              \
      FAIL();                                                                                      \
    }                                                                                              \
  } while (0)

  keep_pool_memory(g->device);
  CK(cudaStreamCreateWithFlags(&g->stream, cudaStreamNonBlocking));
  CK(cudaStreamCreateWithFlags(&g->copy_stream, cudaStreamNonBlocking));
  for (int k = 0; k < kMaxCopyGroups; k++) CK(cudaEventCreateWithFlags(&g->ev_ready[k], cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&g->ev_free, cudaEventDisableTiming));
  CK(cudaEventCreateWithFlags(&g->ev_fork, cudaEventDisableTiming));
  for (int i = 0; i < MAX_OUTPUTS; i++) {
    CK(cudaStreamCreateWithFlags(&g->prod[i].own_stream, cudaStreamNonBlocking));
    g->prod[i].stream = g->prod[i].own_stream;
    CK(cudaEventCreateWithFlags(&g->prod[i].ev_join, cudaEventDisableTiming));
  }

  const size_t blk_bytes = (size_t)ctx->Ntpb * ctx->Np * ctx->Nc * 2 * (ctx->Nbps / 8);
  // Host input blocks.  Default (cached) pinned memory: on a Grace host the
  // copy engines read write-combined pages at less than half the rate.
  if (!ctx->h_blkbufs) {
    g->caller_managed = false;
    ctx->h_blkbufs = (char**)calloc(ctx->Nb_host, sizeof(char*));
    if (!ctx->h_blkbufs) FAIL();
    for (unsigned i = 0; i < ctx->Nb_host; i++)
      CK(pinned_alloc((void**)&ctx->h_blkbufs[i], blk_bytes));
  } else {
    g->caller_managed = true;
    g->locked_here.assign(ctx->Nb_host, 0);
    for (unsigned i = 0; i < ctx->Nb_host; i++) {
      // blocks the caller already page-locked (cudaHostAlloc) are used as they are
      cudaPointerAttributes pa;
      const bool pinned = cudaPointerGetAttributes(&pa, ctx->h_blkbufs[i]) == cudaSuccess &&
                          pa.type == cudaMemoryTypeHost;
      cudaGetLastError();
      if (!pinned) {
        CK(cudaHostRegister(ctx->h_blkbufs[i], blk_bytes, cudaHostRegisterDefault));
        g->locked_here[i] = 1;
      }
      g->registered = i + 1;
    }
  }

  // Device input buffer.
  g->in_bytes = blk_bytes * ctx->Nb;
  if (dev_alloc(g, &g->d_in, g->in_bytes)) FAIL();
  CK(cudaMemsetAsync(g->d_in, 0, g->in_bytes, g->stream));
  if (expanded) {
    g->in4_bytes = g->in_bytes / 2;
    if (dev_alloc(g, &g->d_in4, g->in4_bytes)) FAIL();
  }

  // Antenna weights.
  if (ctx->incoherently_sum) {
    if (dev_alloc(g, &g->d_aws, ctx->Nant * sizeof(float))) FAIL();
    std::vector<float> w(ctx->Nant);
    for (unsigned a = 0; a < ctx->Nant; a++) w[a] = ctx->Naws == 1 ? ctx->Aws[0] : ctx->Aws[a];
    if (ctx->Naws == 1 && ctx->Nant > 1)
      printf("Using the single antenna-weight (%f) for all antennas in the incoherent-sum.\n", ctx->Aws[0]);
    CK(cudaMemcpy(g->d_aws, w.data(), ctx->Nant * sizeof(float), cudaMemcpyHostToDevice));
  }

  // Products.  The kernels work on the integer codes; the SNORM scale
  // (1/127 or 1/32767 per component) is applied to the quadratic products.
  const float snorm_d = ctx->Nbps == 16 ? 32767.0f : 127.0f;
  const float scale = 1.0f / (snorm_d * snorm_d);
  for (unsigned i = 0; i < ctx->No; i++) {
    Product& P = g->prod[i];
    const rawspec_gb300_tune tune = tune_for(ctx, (int)i);
    const int target_ctas = target_ctas_for(g->sm_count, tune);
    P.N = (int)ctx->Nts[i];
    P.logN = ilog2u(ctx->Nts[i]);
    P.np = abs(ctx->Npolout[i]);
    P.Na = ctx->Nas[i];
    derived(ctx, (int)i, &P.Nss, &P.Nis, &P.Nd);
    const int pol = P.np == 1 ? POL_TP : ctx->Npolout[i];
    const int M = (int)(P.Nis > 1 ? P.Nss : P.Na);
    const int upc = (int)(P.Nis > 1 ? 1 : P.Nss / P.Na);

    CK(pinned_alloc((void**)&ctx->h_pwrbuf[i], ctx->h_pwrbuf_size[i]));
    P.out_bytes = ctx->h_pwrbuf_size[i];
    if (dev_alloc(g, &P.d_out, P.out_bytes)) FAIL();
    CK(cudaMemsetAsync(P.d_out, 0, P.out_bytes, g->stream));
    P.kahan = kahan_wanted(P.Na, P.Nis);
    if (P.kahan) {
      if (dev_alloc(g, &P.d_stage, P.out_bytes)) FAIL();
      if (dev_alloc(g, &P.d_comp, P.out_bytes)) FAIL();
      CK(cudaMemsetAsync(P.d_comp, 0, P.out_bytes, g->stream));
    }
    if (ctx->incoherently_sum) {
      P.ics_bytes = ctx->h_pwrbuf_size[i] / ctx->Nant;
      CK(pinned_alloc((void**)&ctx->h_icsbuf[i], P.ics_bytes));
      if (dev_alloc(g, &P.d_ics, P.ics_bytes)) FAIL();
      CK(cudaMemsetAsync(P.d_ics, 0, P.ics_bytes, g->stream));
    }

    P.large = P.logN > 12;
    P.tc = !P.large && tensor_dft_wanted(P.logN, pol, tune) && tc_supported(P.logN, g->fmt, (int)ctx->Np, pol, M);
    if (P.tc) {
      TcLaunch& L = P.tl;
      L.logN = P.logN;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      L.chan_stride = (long long)ctx->Nb * ctx->Ntpb;
      L.in = g->d_in;
      L.out = P.d_out;
      L.conj = ctx->input_conjugated ? 1 : 0;
      L.scale = scale;
      size_t pf = 0;
      if (tc_configure(L, &pf, std::min<int>(kMaxCopyGroups, (int)ctx->Nc))) {
        fprintf(stderr, "tensor-core DFT kernel unavailable for FFT length %d\n", P.N);
        FAIL();
      }
      if (pf && dev_alloc(g, &P.d_partial, pf * sizeof(float))) FAIL();
      const size_t tb = tc_table_bytes(P.logN);
      if (dev_alloc(g, &P.d_tw, (tb + 15) & ~size_t(15))) FAIL();
      CK(tc_table_fill(P.d_tw, P.logN, g->stream));
      L.tab = P.d_tw;
      if (dev_alloc(g, &P.d_ctl, sizeof(int))) FAIL();
      CK(cudaMemsetAsync(P.d_ctl, 0, sizeof(int), g->stream));
      CK(pinned_alloc((void**)&P.h_err, sizeof(int)));
      *P.h_err = 0;
      L.err = P.d_ctl;
    } else if (!P.large) {
      SmallLaunch& L = P.sl;
      L.logN = P.logN;
      L.fmt = g->fmt;
      L.nv = (int)ctx->Np;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      L.chan_stride = (long long)ctx->Nb * ctx->Ntpb;
      L.in = g->d_in;
      L.out = P.d_out;
      L.conj = ctx->input_conjugated ? 1 : 0;
      size_t pf = 0;
      if (small_configure(L, target_ctas, &pf, std::min<int>(kMaxCopyGroups, (int)ctx->Nc))) {
        fprintf(stderr, "unsupported FFT length %d\n", P.N);
        FAIL();
      }
      if (pf && dev_alloc(g, &P.d_partial, pf * sizeof(float))) FAIL();
      const int R = small_radix(P.logN, pol);
      const size_t ntw = (size_t)std::max(stockham_table_size(P.N, R), 1);
      if (dev_alloc(g, &P.d_tw, ntw * sizeof(float2))) FAIL();
      CK(stockham_twiddle_fill(P.d_tw, P.N, R, g->stream));
      L.tw = P.d_tw;
      L.scale = scale;
      CK(small_prepare(L));
    } else {
      LargeLaunch& L = P.ll;
      L.logN = P.logN;
      L.fmt = g->fmt;
      L.nv = (int)ctx->Np;
      L.pol = pol;
      L.Nc = (int)ctx->Nc;
      L.Nss = (int)P.Nss;
      L.M = M;
      L.units_per_chan = upc;
      L.n_units = (int)ctx->Nc * upc;
      L.chan_stride = (long long)ctx->Nb * ctx->Ntpb;
      L.in = g->d_in;
      L.out = P.d_out;
      L.conj = ctx->input_conjugated ? 1 : 0;
      size_t sf = 0, pf = 0;
      if (large_configure(L, target_ctas, &sf, &pf)) {
        fprintf(stderr, "unsupported FFT length %d\n", P.N);
        FAIL();
      }
      if (large_fused_supported(L)) {
        P.fused = true;
        L.S = (int)ctx->Nc * (int)P.Nss;
        CK(large_fused_plan(L));
        apply_fused_tune(L, tune);
        // slots in use: slab mod ring over at most S slabs
        sf = (size_t)std::min(L.ring, L.S) * L.nv * ((size_t)1 << L.logN);
        pf = 0;
        const size_t nctl = (size_t)large_fused_ctl_ints(L);
        if (dev_alloc(g, &P.d_ctl, nctl * sizeof(int))) FAIL();
        CK(cudaMemsetAsync(P.d_ctl, 0, nctl * sizeof(int), g->stream));
        CK(pinned_alloc((void**)&P.h_err, sizeof(int)));
        *P.h_err = 0;
        L.ctl = P.d_ctl;
      }
      if (sf && dev_alloc(g, &P.d_scratch, sf * sizeof(float2))) FAIL();
      if (pf && dev_alloc(g, &P.d_partial, pf * sizeof(float))) FAIL();
      const int n1 = 1 << L.logN1, n2 = 1 << L.logN2;
      const int RA = P.fused ? large_fused_col_radix() : large_pass_a_radix();
      const int RB = P.fused ? large_fused_row_radix(pol) : large_pass_b_radix(pol);
      // tables at 256-byte aligned offsets (the fused kernel copies twM and
      // twJ with the tensor copy engine)
      auto al = [](size_t n) { return (n + 31) & ~size_t(31); };
      const size_t ta = (size_t)stockham_table_size(n2, RA), tb = (size_t)stockham_table_size(n1, RB);
      const size_t nlo = (size_t)1 << L.h, nhi = (size_t)1 << (L.logN - L.h), nm = (size_t)RA * n1;
      const size_t nj = P.fused ? (size_t)large_fused_twj_entries(L) : 0;
      const size_t o_tb = al(ta), o_lo = o_tb + al(tb), o_hi = o_lo + al(nlo), o_m = o_hi + al(nhi);
      const size_t o_j = o_m + al(nm);
      if (dev_alloc(g, &P.d_tw, (o_j + nj) * sizeof(float2))) FAIL();
      L.twN2 = P.d_tw;
      L.twN1 = P.d_tw + o_tb;
      L.twLo = P.d_tw + o_lo;
      L.twHi = P.d_tw + o_hi;
      L.twM = P.d_tw + o_m;
      L.twJ = P.fused ? P.d_tw + o_j : nullptr;
      L.scale = scale;
      CK(stockham_twiddle_fill(P.d_tw, n2, RA, g->stream));
      CK(stockham_twiddle_fill(P.d_tw + o_tb, n1, RB, g->stream));
      CK(twiddle_fill(P.d_tw + o_lo, (long long)nlo, (long long)P.N, 1, g->stream));
      CK(twiddle_fill(P.d_tw + o_hi, (long long)nhi, (long long)P.N, (long long)nlo, g->stream));
      CK(passa_twiddle_fill(P.d_tw + o_m, n1, RA, (long long)(n2 / RA), (long long)P.N, g->stream));
      if (P.fused) CK(passa_twiddle_fill(P.d_tw + o_j, n1, n2 / RA, 1, (long long)P.N, g->stream));
      if (P.fused) {
        if (P.kahan) {  // the same maps over the staging plane; its output map is kept
          LargeLaunch Ls = L;
          Ls.out = P.d_stage;
          CK(large_fused_prepare(Ls));
          P.tmap_stage = Ls.tmap_out;
        }
        CK(large_fused_prepare(L));
      } else {
        CK(large_prepare(L));
      }
    }
  }
  for (unsigned i = 0; i < ctx->No; i++) {
    g->prod[i].tl.partial = g->prod[i].d_partial;
    g->prod[i].sl.partial = g->prod[i].d_partial;
    g->prod[i].ll.partial = g->prod[i].d_partial;
    g->prod[i].ll.scratch = g->prod[i].d_scratch;
  }
  CK(cudaStreamSynchronize(g->stream));
  g->inbuf_count = 0;
  return 0;
#undef CK
#undef FAIL
}

void rawspec_cleanup(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  // nothing may still use the buffers: every stream of the context drains first
  if (g) {
    if (g->stream) cudaStreamSynchronize(g->stream);
    if (g->copy_stream) cudaStreamSynchronize(g->copy_stream);
    for (int i = 0; i < MAX_OUTPUTS; i++)
      if (g->prod[i].own_stream) cudaStreamSynchronize(g->prod[i].own_stream);
  }
  for (int i = 0; i < MAX_OUTPUTS; i++) {
    if (ctx->h_pwrbuf[i]) {
      pinned_free(ctx->h_pwrbuf[i], ctx->h_pwrbuf_size[i]);
      ctx->h_pwrbuf[i] = nullptr;
    }
    if (ctx->h_icsbuf[i]) {
      pinned_free(ctx->h_icsbuf[i], g ? g->prod[i].ics_bytes : ctx->h_pwrbuf_size[i] / std::max(1u, ctx->Nant));
      ctx->h_icsbuf[i] = nullptr;
    }
  }
  if (!g) return;
  const size_t blk_bytes = (size_t)ctx->Ntpb * ctx->Np * ctx->Nc * 2 * (ctx->Nbps / 8);
  if (g->caller_managed) {
    for (unsigned i = 0; i < g->registered; i++)
      if (g->locked_here[i]) cudaHostUnregister(ctx->h_blkbufs[i]);
  } else if (ctx->h_blkbufs) {
    for (unsigned i = 0; i < ctx->Nb_host; i++)
      if (ctx->h_blkbufs[i]) pinned_free(ctx->h_blkbufs[i], blk_bytes);
    free(ctx->h_blkbufs);
    ctx->h_blkbufs = nullptr;
  }
  auto dfree = [&](void* p) {
    if (p) cudaFreeAsync(p, g->stream);
  };
  dfree(g->d_in);
  dfree(g->d_in4);
  dfree(g->d_aws);
  for (int i = 0; i < MAX_OUTPUTS; i++) {
    dfree(g->prod[i].d_out);
    dfree(g->prod[i].d_ics);
    dfree(g->prod[i].d_tw);
    dfree(g->prod[i].d_ctl);
    pinned_free(g->prod[i].h_err, sizeof(int));
    dfree(g->prod[i].d_partial);
    dfree(g->prod[i].d_scratch);
    dfree(g->prod[i].d_stage);
    dfree(g->prod[i].d_comp);
    if (g->prod[i].own_stream) cudaStreamDestroy(g->prod[i].own_stream);
    if (g->prod[i].ev_join) cudaEventDestroy(g->prod[i].ev_join);
  }
  if (g->stream) cudaStreamSynchronize(g->stream);
  for (auto& kv : g->graphs)
    if (kv.second.exec) cudaGraphExecDestroy(kv.second.exec);
  if (g->ev_fork) cudaEventDestroy(g->ev_fork);
  for (auto& p : g->pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : g->free_events) cudaEventDestroy(e);
  if (g->copy_stream) cudaStreamDestroy(g->copy_stream);
  for (int k = 0; k < kMaxCopyGroups; k++)
    if (g->ev_ready[k]) cudaEventDestroy(g->ev_ready[k]);
  if (g->ev_free) cudaEventDestroy(g->ev_free);
  if (g->stream) cudaStreamDestroy(g->stream);
  delete g;
  ctx->gpu_ctx = nullptr;
}

int rawspec_copy_blocks_to_gpu(rawspec_context* ctx, off_t src_idx, off_t dst_idx, size_t num_blocks) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  const size_t blk_chan = (size_t)ctx->Ntpb * ctx->Np * 2 * (ctx->Nbps / 8);
  {
    ProfScope ps(g, RAWSPEC_GB300_K_H2D);
    for (size_t b = 0; b < num_blocks; b++) {
      const off_t sblk = (src_idx + (off_t)b) % ctx->Nb_host;
      const off_t dblk = (dst_idx + (off_t)b) % ctx->Nb;
      RSG_CUDA(cudaMemcpy2DAsync((char*)g->d_in + dblk * blk_chan, ctx->Nb * blk_chan, ctx->h_blkbufs[sblk],
                                 blk_chan, blk_chan, ctx->Nc, cudaMemcpyHostToDevice, g->stream));
    }
  }
  RSG_CUDA(cudaStreamSynchronize(g->stream));
  return 0;
}

int rawspec_copy_blocks_to_gpu_expanding_complex4(rawspec_context* ctx, off_t src_idx, off_t dst_idx,
                                                  size_t num_blocks) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  if (num_blocks > ctx->Nb) {
    fprintf(stderr, "%s: num_blocks (%zu) > Nb (%u)\n", __FUNCTION__, num_blocks, ctx->Nb);
    return 1;
  }
  const size_t blk_packed = (size_t)ctx->Ntpb * ctx->Np;  // bytes per channel per block
  if (!g->d_in4) {
    g->in4_bytes = g->in_bytes / 2;
    if (dev_alloc(g, &g->d_in4, g->in4_bytes)) return 1;
  }
  {
    ProfScope ps(g, RAWSPEC_GB300_K_H2D);
    for (size_t b = 0; b < num_blocks; b++) {
      const off_t sblk = (src_idx + (off_t)b) % ctx->Nb_host;
      const off_t dblk = (dst_idx + (off_t)b) % ctx->Nb;
      RSG_CUDA(cudaMemcpy2DAsync(g->d_in4 + dblk * blk_packed, ctx->Nb * blk_packed, ctx->h_blkbufs[sblk],
                                 blk_packed, blk_packed, ctx->Nc, cudaMemcpyHostToDevice, g->stream));
    }
  }
  Expand4Launch E;
  E.packed = g->d_in4;
  E.out = reinterpret_cast<int8_t*>(g->d_in);
  E.Nc = (int)ctx->Nc;
  E.Nb = (int)ctx->Nb;
  E.blk_bytes_packed = (long long)blk_packed;
  E.dst_block = (int)(dst_idx % ctx->Nb);
  E.num_blocks = (int)num_blocks;
  {
    ProfScope ps(g, RAWSPEC_GB300_K_EXPAND4);
    RSG_CUDA(expand4_launch(E, g->stream));
    g->launches++;
  }
  RSG_CUDA(cudaStreamSynchronize(g->stream));
  return 0;
}

int rawspec_zero_blocks_to_gpu(rawspec_context* ctx, off_t dst_idx, size_t num_blocks) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  const size_t blk_chan = (size_t)ctx->Ntpb * ctx->Np * 2 * (ctx->Nbps / 8);
  for (size_t b = 0; b < num_blocks; b++) {
    const off_t dblk = (dst_idx + (off_t)b) % ctx->Nb;
    RSG_CUDA(cudaMemset2DAsync((char*)g->d_in + dblk * blk_chan, ctx->Nb * blk_chan, 0, blk_chan, ctx->Nc,
                               g->stream));
  }
  RSG_CUDA(cudaStreamSynchronize(g->stream));
  return 0;
}

int rawspec_start_processing(rawspec_context* ctx, int fft_dir) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  if (g->profiling || !graphs_wanted(g)) return process_buffer(ctx, g, fft_dir, 1, nullptr);
  // the pattern of the buffer about to be processed (inbuf_count + 1)
  const unsigned next = g->inbuf_count + 1;
  unsigned long long key = (fft_dir <= 0 ? 1ull : 0ull) | (ctx->dump_callback ? 2ull : 0ull);
  for (unsigned i = 0; i < ctx->No; i++) {
    const Product& P = g->prod[i];
    const unsigned long long m = ((next - 1) % P.Nis == 0 ? 0ull : 1ull) | (next % P.Nis == 0 ? 2ull : 0ull);
    key |= m << (2 + 2 * i);
  }
  auto it = g->graphs.find(key);
  if (it == g->graphs.end()) {
    if (g->graphs.size() >= kMaxGraphs) return process_buffer(ctx, g, fft_dir, 1, nullptr);
    // capture the launches of this pattern (nothing runs while capturing)
    const unsigned saved_count = g->inbuf_count;
    const unsigned long long saved_launches = g->launches;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
    bool ok = cudaStreamBeginCapture(g->stream, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
      const int rc = process_buffer(ctx, g, fft_dir, 1, nullptr);
      ok = cudaStreamEndCapture(g->stream, &graph) == cudaSuccess && rc == 0 && graph &&
           cudaGraphInstantiate(&exec, graph, 0) == cudaSuccess;
    }
    if (graph) cudaGraphDestroy(graph);
    const unsigned long long launches = g->launches - saved_launches;
    g->inbuf_count = saved_count;
    g->launches = saved_launches;
    if (!ok) {
      cudaGetLastError();
      if (exec) cudaGraphExecDestroy(exec);
      g->graphs[key] = GpuCtx::Graph{nullptr, 0};  // this pattern is launched directly from now on
      return process_buffer(ctx, g, fft_dir, 1, nullptr);
    }
    it = g->graphs.emplace(key, GpuCtx::Graph{exec, launches}).first;
  }
  if (!it->second.exec) return process_buffer(ctx, g, fft_dir, 1, nullptr);
  g->inbuf_count++;
  g->launches += it->second.launches;
  RSG_CUDA(cudaGraphLaunch(it->second.exec, g->stream));
  return 0;
}

// One buffer of each of several contexts (e.g. the jobs of a server): each
// context's work as rawspec_start_processing queues it, except that the
// k_small launches of the contexts that share a kernel configuration run as
// one grid.  Contexts on different devices, or with profiling on, are
// processed one after another instead.
int rawspec_gb300_start_processing_group(rawspec_context* const* ctxs, const int* fft_dirs, int n) {
  if (!ctxs || !fft_dirs || n < 1) return 1;
  GpuCtx* g0 = G(ctxs[0]);
  if (!g0) return 1;
  bool plain = n == 1;
  for (int k = 0; k < n; k++) {
    GpuCtx* g = ctxs[k] ? G(ctxs[k]) : nullptr;
    if (!g) return 1;
    for (int m = 0; m < k; m++)
      if (ctxs[m] == ctxs[k]) return 1;
    if (g->device != g0->device || g->profiling) plain = true;
  }
  if (plain) {
    for (int k = 0; k < n; k++)
      if (rawspec_start_processing(ctxs[k], fft_dirs[k])) return 1;
    return 0;
  }
  std::vector<DeferredSmall> d;
  for (int k = 0; k < n; k++)
    if (buffer_launches(ctxs[k], G(ctxs[k]), fft_dirs[k], 1, nullptr, &d)) return 1;
  if (launch_deferred(d)) return 1;
  for (int k = 0; k < n; k++)
    if (buffer_finish(ctxs[k], G(ctxs[k]))) return 1;
  return 0;
}

// The copy of a full buffer is split into channel groups on a copy stream;
// the kernels of group k start as soon as its copy has landed, so the
// host-to-device transfer overlaps the processing.  The call returns, like
// the reference's, once the host blocks may be reused.
int rawspec_copy_blocks_to_gpu_and_start_processing(rawspec_context* ctx, size_t num_blocks, char expand4bps_to8bps,
                                                    int fft_dir) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  const int ngroups = std::min<int>(kMaxCopyGroups, (int)ctx->Nc);
  if (num_blocks != ctx->Nb || ngroups < 2 || g->in_bytes < kMinPipelinedBytes) {
    const int rc = expand4bps_to8bps ? rawspec_copy_blocks_to_gpu_expanding_complex4(ctx, 0, 0, num_blocks)
                                     : rawspec_copy_blocks_to_gpu(ctx, 0, 0, num_blocks);
    if (rc) return rc;
    return rawspec_start_processing(ctx, fft_dir);
  }
  const bool packed = expand4bps_to8bps != 0;
  if (packed && !g->d_in4) {
    g->in4_bytes = g->in_bytes / 2;
    if (dev_alloc(g, &g->d_in4, g->in4_bytes)) return 1;
  }
  // bytes per channel per block in the host block and in the device buffer
  const size_t row = packed ? (size_t)ctx->Ntpb * ctx->Np : (size_t)ctx->Ntpb * ctx->Np * 2 * (ctx->Nbps / 8);
  char* dev = packed ? reinterpret_cast<char*>(g->d_in4) : reinterpret_cast<char*>(g->d_in);
  // The previous buffer's processing must be finished with the input.
  RSG_CUDA(cudaEventRecord(g->ev_free, g->stream));
  RSG_CUDA(cudaStreamWaitEvent(g->copy_stream, g->ev_free, 0));
  for (int grp = 0; grp < ngroups; grp++) {
    const size_t c0 = (size_t)grp * ctx->Nc / ngroups;
    const size_t c1 = (size_t)(grp + 1) * ctx->Nc / ngroups;
    for (size_t b = 0; b < num_blocks; b++) {
      RSG_CUDA(cudaMemcpy2DAsync(dev + c0 * ctx->Nb * row + b * row, ctx->Nb * row, ctx->h_blkbufs[b] + c0 * row, row,
                                 row, c1 - c0, cudaMemcpyHostToDevice, g->copy_stream));
    }
    if (packed) {  // the group's 4-bit samples are expanded right behind its copy
      Expand4Launch E;
      E.packed = g->d_in4;
      E.out = reinterpret_cast<int8_t*>(g->d_in);
      E.Nc = (int)ctx->Nc;
      E.Nb = (int)ctx->Nb;
      E.blk_bytes_packed = (long long)row;
      E.dst_block = 0;
      E.num_blocks = (int)num_blocks;
      E.c0 = (int)c0;
      E.nch = (int)(c1 - c0);
      ProfScope ps(g, RAWSPEC_GB300_K_EXPAND4, g->copy_stream);
      RSG_CUDA(expand4_launch(E, g->copy_stream));
      g->launches++;
    }
    RSG_CUDA(cudaEventRecord(g->ev_ready[grp], g->copy_stream));
  }
  if (process_buffer(ctx, g, fft_dir, ngroups, g->ev_ready)) return 1;
  RSG_CUDA(cudaStreamSynchronize(g->copy_stream));
  return 0;
}

int rawspec_reset_integration(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  rawspec_wait_for_completion(ctx);
  for (unsigned i = 0; i < ctx->No; i++) {
    RSG_CUDA(cudaMemsetAsync(g->prod[i].d_out, 0, g->prod[i].out_bytes, g->stream));
    if (g->prod[i].d_ics) RSG_CUDA(cudaMemsetAsync(g->prod[i].d_ics, 0, g->prod[i].ics_bytes, g->stream));
  }
  RSG_CUDA(cudaStreamSynchronize(g->stream));
  g->inbuf_count = 0;
  return 0;
}

unsigned int rawspec_check_for_completion(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  if (!g) return 0;
  return cudaStreamQuery(g->stream) == cudaSuccess ? 1u : 0u;
}

int rawspec_wait_for_completion(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  if (ctx->dump_callback)
    for (unsigned i = 0; i < ctx->No; i++) RSG_CUDA(cudaLaunchHostFunc(g->stream, pre_dump_fn, &g->cb[i]));
  if (cudaStreamSynchronize(g->stream) != cudaSuccess) return 1;
  for (unsigned i = 0; i < ctx->No; i++) {
    if (!g->prod[i].h_err) continue;
    const int err = *g->prod[i].h_err;  // copied behind every fused or tc launch, ordered before the join
    if (err) {
      if (g->prod[i].tc)
        fprintf(stderr, "rawspec: product %u: a bounded wait for the tensor cores timed out\n", i);
      else
        fprintf(stderr, "rawspec: product %u: a bounded wait of the fused FFT kernel timed out (code %d: 1 ring "
                        "slot, 2 column tiles, 3 stage copy)\n", i, err);
      return 1;
    }
  }
  if (ctx->exit_soon)
    fprintf(stderr, "*** rawspec_wait_for_completion detected exit_soon enabled.\n*** Cannot continue!\n");
  return (int)ctx->exit_soon;
}

// ---------------------------------------------------------------------------
// Extensions.
// ---------------------------------------------------------------------------
void* rawspec_gb300_stream(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  return g ? (void*)g->stream : nullptr;
}

void* rawspec_gb300_device_input(rawspec_context* ctx, size_t* bytes) {
  GpuCtx* g = G(ctx);
  if (!g) return nullptr;
  if (bytes) *bytes = g->in_bytes;
  return g->d_in;
}

int rawspec_gb300_set_profiling(rawspec_context* ctx, int enable) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  g->profiling = enable != 0;
  return 0;
}

int rawspec_gb300_profile(rawspec_context* ctx, int kernel_class, double* total_ms, unsigned long long* launches) {
  GpuCtx* g = G(ctx);
  if (!g || kernel_class < 0 || kernel_class >= RAWSPEC_GB300_K_COUNT) return 1;
  if (cudaStreamSynchronize(g->stream) != cudaSuccess) return 1;
  collect_profile(g);
  if (total_ms) *total_ms = g->prof_ms[kernel_class];
  if (launches) *launches = g->prof_n[kernel_class];
  return 0;
}

int rawspec_gb300_reset_profile(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  if (!g) return 1;
  if (cudaStreamSynchronize(g->stream) != cudaSuccess) return 1;
  collect_profile(g);
  for (int k = 0; k < RAWSPEC_GB300_K_COUNT; k++) {
    g->prof_ms[k] = 0;
    g->prof_n[k] = 0;
  }
  return 0;
}

unsigned long long rawspec_gb300_shared_launches(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  return g ? g->shared_launches : 0;
}

unsigned long long rawspec_gb300_kernel_launches(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  return g ? g->launches : 0;
}

size_t rawspec_gb300_device_bytes(rawspec_context* ctx) {
  GpuCtx* g = G(ctx);
  return g ? g->device_bytes : 0;
}

int rawspec_gb300_device_bytes_estimate(const rawspec_context* ctx, size_t* bytes) {
  if (!ctx || !bytes) return 1;
  rawspec_context c = *ctx;  // validation normalises fields of its own copy
  bool expanded = false;
  if (validate_impl(&c, &expanded)) return 1;
  int dev = 0, sms = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) return 1;
  if (dev != c.gpu_index && cudaSetDevice(c.gpu_index) != cudaSuccess) return 1;
  const bool ok = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c.gpu_index) == cudaSuccess &&
                  plan_device_bytes(&c, expanded, sms, bytes) == 0;
  if (dev != c.gpu_index) cudaSetDevice(dev);
  return ok ? 0 : 1;
}

}  // extern "C"
#pragma GCC visibility pop
