// umma_probe.cu -- test helper: one CTA copies a host-built shared-memory
// image (two K-major FP16 operands in 8 x 16-byte core matrices), issues the
// library's tcgen05 MMAs on it with the library's descriptors and returns the
// 128 x n FP32 accumulator, so that a test can check the operand layout and
// descriptor encodings against a plain matrix product.
#include <cstdint>
#include <cuda_runtime.h>

#include "tc_ptx.cuh"

namespace {

constexpr int kImage = 163840;  // shared-memory image; any operand read stays inside it
constexpr int kCols = 256;     // tensor-memory columns (the largest n)

__global__ void k_probe(const uint4* img, int img16, int a_off, int b_off, int lbo, int sbo, int n, int k,
                        uint32_t idesc, float* d, int* err) {
  using namespace rsg::tc;
  extern __shared__ __align__(128) unsigned char sm[];
  uint64_t* mbar = reinterpret_cast<uint64_t*>(sm + kImage);
  uint32_t* slot = reinterpret_cast<uint32_t*>(mbar + 2);
  const int tid = threadIdx.x, warp = tid >> 5;
  for (int i = tid; i < kImage / 16; i += 128)
    reinterpret_cast<uint4*>(sm)[i] = i < img16 ? img[i] : make_uint4(0, 0, 0, 0);
  if (tid == 0) mbar_init(mbar, 1);
  if (warp == 0) {
    tmem_alloc(slot, kCols);
    tmem_relinquish();
  }
  fence_proxy_async_smem();
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  const uint32_t tmem = *slot;
  const uint32_t base = smem_u32(sm);
  if (tid == 0) {
    for (int ks = 0; ks < k / 16; ++ks)
      mma_f16(tmem, smem_desc(base + a_off + ks * 2 * lbo, lbo, sbo), smem_desc(base + b_off + ks * 2 * lbo, lbo, sbo),
              idesc, ks > 0 ? 1u : 0u);
    mma_commit(mbar);
  }
  if (!mbar_wait_bounded(mbar, 0, 2000000000ll)) atomicExch(err, 1);
  fence_after_sync();
  const uint32_t trow = tmem + ((uint32_t)(warp * 32) << 16);
  for (int q = 0; q < n / 32; ++q) {
    float a[16], b[16];
    tmem_ld16x2(trow + 32 * q, trow + 32 * q + 16, a, b);
    for (int i = 0; i < 16; ++i) {
      d[tid * n + 32 * q + i] = a[i];
      d[tid * n + 32 * q + 16 + i] = b[i];
    }
  }
  fence_before_sync();
  __syncthreads();
  fence_after_sync();
  if (warp == 0) tmem_dealloc(tmem, kCols);
}

}  // namespace

// img: the operand image (img_bytes <= 163840, a multiple of 16); A (128 x k)
// at a_off, B (n x k) at b_off; n a multiple of 32 in [32, 256], k a multiple
// of 16.  out: 128 x n floats.  Returns 0, or a nonzero step number.
extern "C" int umma_probe(const void* img, int img_bytes, int a_off, int b_off, int lbo, int sbo, int n, int k,
                          float* out) {
  if (img_bytes > kImage || img_bytes % 16 || n % 32 || n < 32 || n > kCols || k % 16) return 1;
  void* d_img = nullptr;
  float* d_out = nullptr;
  int* d_err = nullptr;
  int err = 0;
  if (cudaMalloc(&d_img, img_bytes) != cudaSuccess) return 2;
  if (cudaMalloc(&d_out, sizeof(float) * 128 * n) != cudaSuccess) return 3;
  if (cudaMalloc(&d_err, sizeof(int)) != cudaSuccess) return 4;
  if (cudaMemcpy(d_img, img, img_bytes, cudaMemcpyHostToDevice) != cudaSuccess) return 5;
  if (cudaMemset(d_err, 0, sizeof(int)) != cudaSuccess) return 6;
  const int smem = kImage + 32;
  if (cudaFuncSetAttribute(k_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, smem) != cudaSuccess) return 7;
  k_probe<<<1, 128, smem>>>(static_cast<const uint4*>(d_img), img_bytes / 16, a_off, b_off, lbo, sbo, n, k,
                            rsg::tc::idesc_f16_f32(128, n), d_out, d_err);
  if (cudaGetLastError() != cudaSuccess) return 8;
  if (cudaDeviceSynchronize() != cudaSuccess) return 9;
  if (cudaMemcpy(out, d_out, sizeof(float) * 128 * n, cudaMemcpyDeviceToHost) != cudaSuccess) return 10;
  if (cudaMemcpy(&err, d_err, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) return 11;
  cudaFree(d_img);
  cudaFree(d_out);
  cudaFree(d_err);
  return err ? 12 : 0;
}
