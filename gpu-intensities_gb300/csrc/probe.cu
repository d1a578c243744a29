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

// ---------------------------------------------------------------- tcgen05 rate
namespace {
__device__ __forceinline__ uint32_t probe_sptr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
// K-major 32-byte-row tile descriptor (32-byte swizzle), as the split GEMM uses.
__device__ __forceinline__ uint64_t probe_desc(uint32_t addr) {
  return (uint64_t)((addr >> 4) & 0x3FFF) | ((uint64_t)1 << 16) | ((uint64_t)16 << 32) |
         ((uint64_t)1 << 46) | ((uint64_t)6 << 61);
}
// Issues ITERS*9 back-to-back MMAs into one accumulator from zeroed shared
// memory; one thread per CTA times them, the wait for completion is bounded.
template <int N>
__global__ void k_mma_rate(long long* cycles, int iters, int* err) {
  __shared__ __align__(1024) unsigned char sm[128 * 32 + 256 * 32];
  __shared__ uint64_t bar;
  __shared__ uint32_t slot;
  for (int i = threadIdx.x; i < (int)sizeof(sm); i += blockDim.x) sm[i] = 0;
  if (threadIdx.x == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(probe_sptr(&bar)));
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(
        probe_sptr(&slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tmem = slot;
  if (threadIdx.x == 0) {
    const uint32_t idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) |
                           ((uint32_t)(128 >> 4) << 24);
    const uint64_t ad = probe_desc(probe_sptr(sm)), bd = probe_desc(probe_sptr(sm + 128 * 32));
    asm volatile("fence.proxy.async.shared::cta;");
    const long long t0 = clock64();
    for (int it = 0; it < iters; ++it)
#pragma unroll
      for (int j = 0; j < 9; ++j)
        asm volatile(
            "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
            "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(1u));
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            probe_sptr(&bar)));
    uint32_t ok = 0;
    const long long tw = clock64();
    while (!ok && clock64() - tw < 4000000000ll)
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n"
          "selp.u32 %0,1,0,p;\n}"
          : "=r"(ok)
          : "r"(probe_sptr(&bar)));
    if (!ok) atomicExch(err, 1);
    cycles[blockIdx.x] = clock64() - t0;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (threadIdx.x < 32) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem));
  }
}
}  // namespace

extern "C" gi_status gi_measure_mma_cycles(int device, int n, double* cycles) {
  if (!cycles) return GI_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return GI_ERR_CUDA;
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
  long long* d = nullptr;
  int* err = nullptr;
  if (cudaMalloc(&d, sizeof(long long) * sms) != cudaSuccess) return GI_ERR_NOMEM;
  if (cudaMalloc(&err, sizeof(int)) != cudaSuccess) {
    cudaFree(d);
    return GI_ERR_NOMEM;
  }
  cudaMemset(err, 0, sizeof(int));
  const int iters = 2000;
  switch (n) {
    case 32: k_mma_rate<32><<<sms, 128>>>(d, iters, err); break;
    case 48: k_mma_rate<48><<<sms, 128>>>(d, iters, err); break;
    case 64: k_mma_rate<64><<<sms, 128>>>(d, iters, err); break;
    case 96: k_mma_rate<96><<<sms, 128>>>(d, iters, err); break;
    case 128: k_mma_rate<128><<<sms, 128>>>(d, iters, err); break;
    case 256: k_mma_rate<256><<<sms, 128>>>(d, iters, err); break;
    default:
      cudaFree(d);
      cudaFree(err);
      return GI_ERR_ARG;
  }
  const cudaError_t e = cudaDeviceSynchronize();
  long long* h = new long long[sms];
  int herr = 0;
  cudaMemcpy(h, d, sizeof(long long) * sms, cudaMemcpyDeviceToHost);
  cudaMemcpy(&herr, err, sizeof(int), cudaMemcpyDeviceToHost);
  double avg = 0;
  for (int i = 0; i < sms; ++i) avg += (double)h[i];
  delete[] h;
  cudaFree(d);
  cudaFree(err);
  if (e != cudaSuccess) return GI_ERR_CUDA;
  if (herr) return GI_ERR_DEVICE;
  *cycles = avg / sms / (iters * 9.0);
  return GI_OK;
}
