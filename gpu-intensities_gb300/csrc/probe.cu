// FP64 tensor-pipe peak probe (include/gi_probe.h).
#include <cuda_runtime.h>

#include "../../include/gi_probe.h"

namespace {
// Four independent accumulator chains of m8n8k4 DMMA per warp.
__global__ void k_dmma_peak(double* out, int iters) {
  double a = threadIdx.x * 1e-3, b = 1.0000001;
  double d[4][2] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int j = 0; j < 4; ++j)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(d[j][0]), "+d"(d[j][1])
                   : "d"(a), "d"(b));
  }
  double s = 0;
  for (int j = 0; j < 4; ++j) s += d[j][0] + d[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" gi_status gi_measure_fp64_peak(int device, double* tflops) {
  if (!tflops) return GI_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return GI_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  const int blocks = sms * 8, threads = 256, iters = 2000;
  double* out = nullptr;
  if (cudaMalloc(&out, sizeof(double) * blocks * threads) != cudaSuccess) return GI_ERR_NOMEM;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  double best = 0.0;
  for (int rep = 0; rep < 4; ++rep) {
    cudaEventRecord(e0);
    k_dmma_peak<<<blocks, threads>>>(out, iters);
    cudaEventRecord(e1);
    cudaEventSynchronize(e1);
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    // per warp instruction: 8 x 8 x 4 = 256 multiply-adds = 512 flop
    const double flop = 512.0 * 4 * iters * (double)blocks * threads / 32;
    if (rep > 0 && ms > 0) best = flop / (ms * 1e-3) / 1e12 > best ? flop / (ms * 1e-3) / 1e12 : best;
  }
  const cudaError_t err = cudaGetLastError();
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  if (err != cudaSuccess) return GI_ERR_CUDA;
  *tflops = best;
  return GI_OK;
}
