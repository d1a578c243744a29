/* Host-only stand-in for the CUDA runtime header, used solely to compile the
   reference's kernel bodies as plain C++ so that they can run on the CPU as a
   parity pin for the oracle.  Each "launch" is a host loop over thread ids. */
#ifndef GI_REF_CUDA_STUB_H
#define GI_REF_CUDA_STUB_H
#include <cstring>
#include <cstddef>
#define __global__
#define __device__
#define __host__
#define __constant__
#define __shared__
struct gi_ref_dim3 { unsigned x, y, z; };
extern gi_ref_dim3 blockIdx, blockDim, threadIdx, gridDim;
enum { cudaMemcpyHostToDevice = 1 };
template <class T>
inline int cudaMemcpyToSymbol(T& sym, const void* src, size_t n, size_t off, int) {
  std::memcpy(reinterpret_cast<char*>(&sym) + off, src, n);
  return 0;
}
inline void __syncthreads() {}
inline unsigned long long atomicCAS(unsigned long long* a, unsigned long long cmp, unsigned long long v) {
  unsigned long long old = *a; if (old == cmp) *a = v; return old;
}
inline long long __double_as_longlong(double d) { long long r; std::memcpy(&r, &d, 8); return r; }
inline double __longlong_as_double(long long l) { double r; std::memcpy(&r, &l, 8); return r; }
#endif
