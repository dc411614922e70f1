// snorm_probe.cu -- test helper: reads every 8- and 16-bit code through a
// CUDA texture configured like the reference's input texture (pitch 2D,
// signed, cudaReadModeNormalizedFloat, point sampling at integer coordinates;
// rawspec_gpu.cu:845-866, :145-146) and through the library's unpack
// function, so a test can compare the two bit for bit.
#include <cstdint>
#include <cuda_runtime.h>

#include "common.cuh"

__global__ void k_tex(cudaTextureObject_t t, int w, int h, float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < w * h) out[i] = tex2D<float>(t, (float)(i % w), (float)(i / w));
}

__global__ void k_ours8(float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 256) out[i] = rsg::snorm<127>((int)(int8_t)(uint8_t)i);
}

__global__ void k_ours16(float* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < 65536) out[i] = rsg::snorm<32767>((int)(int16_t)(uint16_t)i);
}

static int tex_read(int bits, int w, int h, float* host_out) {
  const size_t esz = bits / 8;
  size_t pitch = 0;
  void* d = nullptr;
  if (cudaMallocPitch(&d, &pitch, w * esz, h) != cudaSuccess) return 1;
  // element i (row-major, w per row) holds code i
  for (int r = 0; r < h; r++) {
    uint8_t row[512];
    for (int x = 0; x < w; x++) {
      const uint32_t code = (uint32_t)(r * w + x);
      if (bits == 8) row[x] = (uint8_t)code;
      else { row[2 * x] = (uint8_t)(code & 0xff); row[2 * x + 1] = (uint8_t)(code >> 8); }
    }
    if (cudaMemcpy((char*)d + r * pitch, row, w * esz, cudaMemcpyHostToDevice) != cudaSuccess) return 2;
  }
  cudaResourceDesc rd = {};
  rd.resType = cudaResourceTypePitch2D;
  rd.res.pitch2D.devPtr = d;
  rd.res.pitch2D.desc.f = cudaChannelFormatKindSigned;
  rd.res.pitch2D.desc.x = bits;
  rd.res.pitch2D.width = w;
  rd.res.pitch2D.height = h;
  rd.res.pitch2D.pitchInBytes = pitch;
  cudaTextureDesc td = {};
  td.readMode = cudaReadModeNormalizedFloat;
  cudaTextureObject_t t = 0;
  if (cudaCreateTextureObject(&t, &rd, &td, nullptr) != cudaSuccess) return 3;
  float* o = nullptr;
  if (cudaMalloc(&o, sizeof(float) * w * h) != cudaSuccess) return 4;
  k_tex<<<(w * h + 255) / 256, 256>>>(t, w, h, o);
  if (cudaMemcpy(host_out, o, sizeof(float) * w * h, cudaMemcpyDeviceToHost) != cudaSuccess) return 5;
  cudaDestroyTextureObject(t);
  cudaFree(o);
  cudaFree(d);
  return 0;
}

extern "C" int snorm_probe(float* tex8, float* ours8, float* tex16, float* ours16) {
  int rc = tex_read(8, 256, 1, tex8);
  if (rc) return rc;
  rc = tex_read(16, 256, 256, tex16);
  if (rc) return 10 + rc;
  float* o = nullptr;
  if (cudaMalloc(&o, sizeof(float) * 65536) != cudaSuccess) return 20;
  k_ours8<<<1, 256>>>(o);
  if (cudaMemcpy(ours8, o, sizeof(float) * 256, cudaMemcpyDeviceToHost) != cudaSuccess) return 21;
  k_ours16<<<256, 256>>>(o);
  if (cudaMemcpy(ours16, o, sizeof(float) * 65536, cudaMemcpyDeviceToHost) != cudaSuccess) return 22;
  cudaFree(o);
  return 0;
}
