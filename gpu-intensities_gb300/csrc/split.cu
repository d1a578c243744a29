// Split-precision GEMMs on the tcgen05 tensor pipe (sm_103a).
//
// C[z][n*ldc + m] = sum_k A[z][m][k] * B[n][k] in FP64 accuracy from bf16
// tensor-core products (an Ozaki-style error-free splitting):
//
//   * every row r of A (and of B) is scaled by 2^-e_r so that |x| < 1/2 and
//     split into s integer digits of w bits,
//       x = sum_p a_p 2^(-w(p+1)) + tail,  a_p in [-2^(w-1), 2^(w-1)],
//       |tail| <= 2^-(ws+1),
//     each digit an exact bf16 integer;
//   * the products a_p * b_q with p + q = d <= s-1 share the weight 2^(-wd);
//     each diagonal d is accumulated in its own fp32 TMEM accumulator, where
//     sums of integer products stay exact while they stay at most 2^24: a
//     product is at most 2^(2w-2) and diagonal d has d+1 of them per k, so
//     for w = 6 and K <= 2048 the sum is at most (d+1) 2^21, exact in the
//     worst case for d <= 7 (the last diagonal of s = 9 carries the weight
//     2^-48, where fp32 rounding is negligible).  Longer K runs in segments
//     of 2048, each adding its FP64 result to the previous ones';
//   * the epilogue combines the diagonals exactly in int64 (Horner in 2^w)
//     and builds the FP64 result scaled by 2^(e_m + e_n - 2w).
//
// Kernels (warp 0 issues TMA loads, one thread of warp 1 issues tcgen05.mma
// for every digit pair of a K slice, the remaining warps read the
// accumulators from TMEM and write FP64):
//   k_split_gemm, k_split_gemm2  plain digit layout: one pass, two passes;
//   k_split_gemm_g   grouped digit layout (four planes per 128-byte TMA row),
//       one or two passes, one 128 x BN tile per CTA;
//   k_split_gemm_gp  the grouped two-pass kernel made persistent over a work
//       list of tiles of several GEMMs (the final-state GEMMs of a group of
//       final blocks), K segments inside;
//   k_slice_rows(_b), k_build_y_digits  FP64 rows -> digit planes (the latter
//       builds the half-ls GEMM's Y rows and cuts them in one pass).
// Every mbarrier wait is bounded by %globaltimer; a timeout sets a device
// error word and the CTA unwinds.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>

#include "split.h"
#include "epilogue.cuh"
#include "items.cuh"
#include "../../include/gi_probe.h"

namespace gi {
namespace {

constexpr int kBM = 128;       // tile rows (MMA M)
constexpr int kBK = 16;        // K elements per stage (32 bytes: SWIZZLE_32B rows)
constexpr int kKSeg = 2048;    // K per launch: the exactness bound of the diagonal sums
constexpr int kStages = 4;
constexpr int kThreads = 192;  // warp 0 TMA, warp 1 MMA, warps 2..5 epilogue
constexpr int kMaxSlices = 10;
constexpr int kDefaultSlices = 9;
constexpr int kDefaultW = 6;

struct SplitShape {
  int s, w, bn;
};

// One-pass tile width: S accumulators of BN columns fit the 512 TMEM columns.
__host__ __device__ constexpr int bn_for(int s) { return s <= 8 ? 64 : 48; }
// At least 120 KB so that one CTA holds an SM (it allocates all 512 TMEM columns).
size_t smem_bytes(int s, int bn) {
  const size_t need = (size_t)kStages * s * (kBM + bn) * kBK * 2 + 1024 /*align*/ + 256;
  return need < (size_t)120 * 1024 ? (size_t)120 * 1024 : need;
}

// ------------------------------------------------------------------ PTX
__device__ __forceinline__ uint32_t sptr(const void* p) {
  return (uint32_t)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(uint64_t* b, int count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(sptr(b)), "r"(count));
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* b, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(sptr(b)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ uint32_t mbar_try(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sptr(b)), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ uint64_t gtimer() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;\n" : "=l"(t));
  return t;
}
// Bounded wait on an mbarrier phase.  Returns false when the CTA is aborting
// (another warp timed out) or this wait exceeded its time limit (then it
// raises the abort itself and records the error).
// `sleep_ns` backs the poll off so that a waiting warp leaves the issue slots of
// its SM sub-partition to the MMA-issuing warp.
// CL: cluster-scope acquire (barriers that the peer CTA of a pair completes).
__device__ __forceinline__ uint32_t mbar_try_cl(uint64_t* b, uint32_t parity);
template <bool CL = false>
__device__ bool mbar_wait(uint64_t* b, uint32_t parity, volatile int* abort_flag, int* err,
                          int code, unsigned sleep_ns = 0) {
  uint64_t t0 = 0;
  for (uint32_t it = 1;; ++it) {
    if (CL ? mbar_try_cl(b, parity) : mbar_try(b, parity)) return true;
    if (sleep_ns) __nanosleep(sleep_ns);
    if ((it & 63) == 0) {
      if (*abort_flag) return false;
      if (*reinterpret_cast<volatile int*>(err)) {  // another CTA timed out: stop waiting
        *abort_flag = 1;
        return false;
      }
      const uint64_t t = gtimer();
      if (t0 == 0) {
        t0 = t;
      } else if (t - t0 > 4000000000ull) {  // 4 s: far beyond any tile's work
        *abort_flag = 1;
        atomicExch(err, code);
        return false;
      }
    }
  }
}
__device__ __forceinline__ void tma_load_3d(void* dst, const CUtensorMap* map, uint64_t* bar,
                                            int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes"
      " [%0], [%1, {%3, %4, %5}], [%2];\n" ::"r"(sptr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(sptr(bar)), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
// The earlier K segments' sum at an output element (K-segmented launches).
// A volatile load: it stays inside its branch, so launches that do not
// accumulate never read C.
__device__ __forceinline__ double ld_acc(const double* p) {
  double v;
  asm volatile("ld.global.f64 %0, [%1];\n" : "=d"(v) : "l"(p) : "memory");
  return v;
}

// v * 2^E for an integer |v| < 2^53 (so the double is exact), built from the
// bits with integer instructions: FP64 throughput is low on this GPU and the
// epilogues convert every output element.  Results outside the normal range
// take ldexp.
__device__ __forceinline__ double scaled_int_body(long long v, int E) {
  if (v == 0) return 0.0;
  const unsigned long long sgn = v < 0 ? (1ull << 63) : 0ull;
  const unsigned long long a = v < 0 ? 0ull - (unsigned long long)v : (unsigned long long)v;
  const int msb = 63 - __clzll((long long)a);
  const int ex = 1023 + msb + E;
  if (msb > 52 || ex <= 0 || ex >= 2047) return ldexp((double)v, E);
  const unsigned long long mant = (a << (52 - msb)) & ((1ull << 52) - 1);
  return __longlong_as_double((long long)(sgn | ((unsigned long long)ex << 52) | mant));
}
// The epilogues call these instead of inlining the conversion: inlined into
// the unrolled column chunks, it made the pass-1 epilogue of the half-ls GEMM
// a long stretch of straight-line code that ran out of the instruction cache
// once per tile (39 us of a 265 us tile, against 21 us called, measured with
// per-tile clock stamps).
__device__ __noinline__ double scaled_int(long long v, int E) { return scaled_int_body(v, E); }
// a0 * 2^ea0 + b0 * 2^eb0 and the same for a second element, in one call (the
// two parts of a two-pass tile's exact sums, added in FP64; the conversions of
// the two elements interleave)
__device__ __noinline__ double2 scaled_pair2(long long a0, int ea0, long long b0, int eb0,
                                             long long a1, int ea1, long long b1, int eb1) {
  double2 r;
  r.x = scaled_int_body(a0, ea0) + scaled_int_body(b0, eb0);
  r.y = scaled_int_body(a1, ea1) + scaled_int_body(b1, eb1);
  return r;
}
// Shared-memory matrix descriptor of a K-major bf16 tile whose rows are 32
// bytes (16 elements) with the 32-byte swizzle: 8-row groups 256 bytes apart.
__device__ __forceinline__ uint64_t sdesc_sw32(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
  d |= (uint64_t)1 << 16;                          // leading byte offset (unused here)
  d |= (uint64_t)((256 >> 4) & 0x3FFF) << 32;      // stride byte offset: 8 rows x 32 B
  d |= (uint64_t)1 << 46;                          // descriptor version (tcgen05)
  d |= (uint64_t)6 << 61;                          // SWIZZLE_32B
  return d;
}
// The same for 128-byte rows with the 128-byte swizzle (8-row groups 1024
// bytes apart).  In the grouped digit layout one such row holds the 16-element
// K slice of four digit planes; the descriptor of plane p of a group starts
// 32 p bytes into the row (the K-step offset inside the swizzle atom).
__device__ __forceinline__ uint64_t sdesc_sw128(uint32_t addr) {
  uint64_t d = 0;
  d |= (uint64_t)((addr >> 4) & 0x3FFF);          // start address
  d |= (uint64_t)1 << 16;                          // leading byte offset (unused here)
  d |= (uint64_t)((1024 >> 4) & 0x3FFF) << 32;     // stride byte offset: 8 rows x 128 B
  d |= (uint64_t)1 << 46;                          // descriptor version (tcgen05)
  d |= (uint64_t)2 << 61;                          // SWIZZLE_128B
  return d;
}
// Instruction descriptor: kind::f16, bf16 x bf16 -> f32, K-major A and B.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
  return (1u << 4)                    // D format f32
         | (1u << 7)                  // A format bf16
         | (1u << 10)                 // B format bf16
         | ((uint32_t)(N >> 3) << 17)  // N
         | ((uint32_t)(M >> 4) << 24); // M
}
__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          sptr(bar))
      : "memory");
}
// ---- the 2-SM pair (cta_group::2): a cluster of two CTAs on one TPC, the
// MMA issued by rank 0 over both CTAs' shared memory (rows 0-127 of A and the
// first half of B's rows from rank 0, the rest from rank 1, at the same
// offsets), each CTA's tensor memory holding its 128 rows of the product.
__device__ __forceinline__ uint32_t cluster_rank() {
  uint32_t r;
  asm volatile("mov.u32 %0, %%cluster_ctarank;\n" : "=r"(r));
  return r;
}
// The shared::cluster address of the same shared-memory location in CTA `rank`.
__device__ __forceinline__ uint32_t mapa_shared(uint32_t addr, uint32_t rank) {
  uint32_t r;
  asm volatile("mapa.shared::cluster.u32 %0, %1, %2;\n" : "=r"(r) : "r"(addr), "r"(rank));
  return r;
}
__device__ __forceinline__ void cluster_sync_all() {
  asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;\n" ::
                   : "memory");
}
// Try-wait with cluster-scope acquire: phases completed by the peer CTA's
// arrivals or TMA bytes.
__device__ __forceinline__ uint32_t mbar_try_cl(uint64_t* b, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n.reg .pred p;\nmbarrier.try_wait.parity.acquire.cluster.shared::cta.b64 p, [%1], %2;\n"
      "selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(sptr(b)), "r"(parity)
      : "memory");
  return ok;
}
__device__ __forceinline__ void mbar_arrive_cl(uint32_t bar_cluster) {
  asm volatile("mbarrier.arrive.release.cluster.shared::cluster.b64 _, [%0];\n" ::"r"(bar_cluster)
               : "memory");
}
// TMA into this CTA's shared memory, completing its bytes on a barrier of
// either CTA of the pair (bar_cluster: a shared::cluster address).
__device__ __forceinline__ void tma_load_3d_pair(void* dst, const CUtensorMap* map,
                                                 uint32_t bar_cluster, int c0, int c1, int c2) {
  asm volatile(
      "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes.cta_group::2"
      " [%0], [%1, {%3, %4, %5}], [%2];\n" ::"r"(sptr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(bar_cluster), "r"(c0), "r"(c1), "r"(c2)
      : "memory");
}
__device__ __forceinline__ void mma_bf16_pair(uint32_t tmem_d, uint64_t a, uint64_t b,
                                              uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::2.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem_d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// Completion of the pair's MMAs so far, on one barrier (own or peer's).
__device__ __forceinline__ void mma_commit_pair(uint32_t bar_cluster) {
  asm volatile(
      "tcgen05.commit.cta_group::2.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
          bar_cluster)
      : "memory");
}
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float* v) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,"
      "%14,%15}, [%16];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
        "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// ------------------------------------------------------------------ GEMM
template <int S, int BN>
__global__ void __launch_bounds__(kThreads, 1)
    k_split_gemm(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                 const int32_t* __restrict__ ea, const int32_t* __restrict__ eb, double* C,
                 int ldc, size_t strideC, int M, int Mpad, int Nc, int K, int w, int nM,
                 int nA, int nN, int GA, int accum, int* err) {
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t kAbytes = S * kBM * kBK * 2;
  constexpr uint32_t kBbytes = S * BN * kBK * 2;
  constexpr uint32_t kStage = kAbytes + kBbytes;
  static_assert(S * BN <= 512, "tensor memory columns");
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + kStages * kStage);
  uint64_t* empty = full + kStages;
  uint64_t* accf = empty + kStages;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(accf + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // Raster: tiles come in groups of GA row tiles (A, across m and z) that stay
  // in L2 while every column tile (B) streams past them once per group.
  const int t = blockIdx.x;  // one tile per CTA, nA * nN tiles (nA = nM * batch)
  const int grp = t / (GA * nN);
  const int r = t - grp * GA * nN;
  const int gsz = min(GA, nA - grp * GA);
  const int ai = grp * GA + r % gsz;
  const int n0 = (r / gsz) * BN, m0 = (ai % nM) * kBM, z = ai / nM;
  const int nk = K / kBK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < kStages; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(accf, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {  // the whole warp allocates all 512 TMEM columns
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                     sptr(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer
      int issued = 0;
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % kStages;
        if (kb >= kStages &&
            !mbar_wait(&empty[st], ((kb / kStages) - 1) & 1, abort_flag, err, 1, 64))
          break;
        unsigned char* sa = smem + st * kStage;
        mbar_expect_tx(&full[st], kStage);
        tma_load_3d(sa, &tmA, &full[st], kb * kBK, z * Mpad + m0, 0);
        tma_load_3d(sa + kAbytes, &tmB, &full[st], kb * kBK, n0, 0);
        issued = kb + 1;
      }
      if (*abort_flag) {
        // let the copies still in flight land before the CTA's smem goes away
        for (int kb = (issued > kStages ? issued - kStages : 0); kb < issued; ++kb) {
          uint64_t t0 = gtimer();
          while (!mbar_try(&full[kb % kStages], (kb / kStages) & 1) && gtimer() - t0 < 1000000000ull) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = idesc_bf16(kBM, BN);
      for (int kb = 0; kb < nk; ++kb) {
        const int st = kb % kStages;
        if (!mbar_wait(&full[st], (kb / kStages) & 1, abort_flag, err, 2)) break;
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t a0 = sptr(smem + st * kStage);
        const uint32_t b0 = a0 + kAbytes;
        {
#pragma unroll
          for (int d = 0; d < S; ++d) {
#pragma unroll
            for (int p = 0; p <= d; ++p) {
              const int q = d - p;
              const uint64_t ad = sdesc_sw32(a0 + p * (kBM * kBK * 2));
              const uint64_t bd = sdesc_sw32(b0 + q * (BN * kBK * 2));
              mma_bf16(tmem + d * BN, ad, bd, idesc, (kb > 0 || p > 0) ? 1u : 0u);
            }
          }
        }
        mma_commit(&empty[st]);  // the stage is free once these MMAs have read it
      }
      mma_commit(accf);  // all accumulators final
      if (*abort_flag) {
        // the MMAs already issued must finish before TMEM is released
        uint64_t t0 = gtimer();
        while (!mbar_try(accf, 0) && gtimer() - t0 < 1000000000ull) {
        }
      }
    }
  } else {
    // epilogue warps 2..5: TMEM lane quarter = warp % 4
    const int q4 = warp & 3;
    const int m = m0 + q4 * 32 + lane;
    const bool ok = mbar_wait(accf, 0, abort_flag, err, 3, 1000);
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if (ok) {
      // The accumulators hold integers (|acc| < 2^31), so the diagonals are
      // combined exactly in two int64 words, hi = sum_{d<kHi} acc_d 2^(w(kHi-1-d))
      // (< 2^53) and lo = sum_{d>=kHi} acc_d 2^(w(S-1-d)); FP64 is used only
      // for the final value hi 2^(E-w(kHi-1)) + lo 2^(E-w(S-1)).
      constexpr int kHi = S < 4 ? S : 4;
      const int emr = (m < M) ? ea[z * Mpad + m] : 0;
      double* Cz = C + (size_t)z * strideC;
      for (int c0 = 0; c0 < BN; c0 += 16) {
        long long hi[16], lo[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) hi[j] = lo[j] = 0;
#pragma unroll
        for (int d = 0; d < S; ++d) {
          float f[16];
          tmem_ld16(tmem + ((uint32_t)(q4 * 32) << 16) + d * BN + c0, f);
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const long long a = (long long)__float2int_rn(f[j]);
            if (d < kHi)
              hi[j] = (hi[j] << w) + a;
            else
              lo[j] = (lo[j] << w) + a;
          }
        }
        if (m < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c0 + j;
            if (n < Nc) {
              const int E = emr + eb[n] - 2 * w;
              const double v = scaled_int(hi[j], E - w * (kHi - 1)) +
                               scaled_int(lo[j], E - w * (S - 1));
              double* dst = Cz + (size_t)n * ldc + m;
              *dst = accum ? ld_acc(dst) + v : v;
            }
          }
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
  }
}

// Two-pass variant.  A 128 x N x 16 bf16 MMA costs max(44, 32 + N/4) cycles on
// this GPU, so it reaches the full tensor rate only from N = 128; one pass with
// all S accumulators in tensor memory limits N to 512/S.  Here pass 0 sweeps K
// for the diagonals [0, D1) and pass 1 sweeps it again for [D1, S), each with
// BN-wide accumulators.  Pass 0's epilogue turns its diagonals (exactly, in
// int64) into FP64 in C; pass 1's epilogue adds its part.  Pass 0 loads only
// the digit planes it uses (p, q < D1).
constexpr int kStages2 = 3;
// Stage of the grouped layout: s/4 four-plane groups of 128-byte rows and s%4
// planes of 32-byte rows, for 128 A rows and bn B rows; 1024-byte aligned so
// every 128-byte-swizzle tile starts on a swizzle period.
__host__ __device__ constexpr uint32_t stage_bytes_g(int s, int bn) {
  return ((uint32_t)((s / 4) * (kBM + bn) * 128 + (s % 4) * (kBM + bn) * 32) + 1023u) / 1024u *
         1024u;
}

template <int S, int BN, int D1>
__global__ void __launch_bounds__(kThreads, 1)
    k_split_gemm2(const __grid_constant__ CUtensorMap tmA, const __grid_constant__ CUtensorMap tmB,
                  const int32_t* __restrict__ ea, const int32_t* __restrict__ eb, double* C,
                  int ldc, size_t strideC, int M, int Mpad, int Nc, int K, int w, int nM, int nA,
                  int nN, int GA, int accum, int* err) {
  static_assert(D1 * BN <= 512 && (S - D1) * BN <= 512, "tensor memory columns");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t kAplane = kBM * kBK * 2, kBplane = BN * kBK * 2;
  constexpr uint32_t kStage = S * (kAplane + kBplane);
  constexpr int ST = kStages2;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST * kStage);
  uint64_t* empty = full + ST;
  uint64_t* accf = empty + ST;  // [2]: a pass's accumulators are final
  uint64_t* tfree = accf + 2;   // pass 0's accumulators have been read
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tfree + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int t = blockIdx.x;
  const int grp = t / (GA * nN);
  const int r = t - grp * GA * nN;
  const int gsz = min(GA, nA - grp * GA);
  const int ai = grp * GA + r % gsz;
  const int n0 = (r / gsz) * BN, m0 = (ai % nM) * kBM, z = ai / nM;
  const int nk = K / kBK;

  if (threadIdx.x == 0) {
    for (int i = 0; i < ST; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&accf[0], 1);
    mbar_init(&accf[1], 1);
    mbar_init(tfree, 128);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                     sptr(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  if (warp == 0) {
    if (lane == 0) {  // TMA producer: both passes, one continuous stage ring
      int issued = 0;
      for (int it = 0; it < 2 * nk; ++it) {
        const int pass = it >= nk, kb = it - pass * nk, st = it % ST;
        const int np = pass ? S : D1;
        if (it >= ST && !mbar_wait(&empty[st], ((it / ST) - 1) & 1, abort_flag, err, 1, 64))
          break;
        unsigned char* sa = smem + st * kStage;
        mbar_expect_tx(&full[st], np * (kAplane + kBplane));
        for (int p = 0; p < np; ++p) {
          tma_load_3d(sa + p * kAplane, &tmA, &full[st], kb * kBK, z * Mpad + m0, p);
          tma_load_3d(sa + S * kAplane + p * kBplane, &tmB, &full[st], kb * kBK, n0, p);
        }
        issued = it + 1;
      }
      if (*abort_flag) {
        for (int it = (issued > ST ? issued - ST : 0); it < issued; ++it) {
          uint64_t t0 = gtimer();
          while (!mbar_try(&full[it % ST], (it / ST) & 1) && gtimer() - t0 < 1000000000ull) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = idesc_bf16(kBM, BN);
      bool ok = true;
      int last = 0;  // the last pass whose MMAs were committed
      for (int pass = 0; pass < 2 && ok; ++pass) {
        last = pass;
        if (pass == 1) {
          ok = mbar_wait(tfree, 0, abort_flag, err, 4);
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          if (!ok) break;
        }
        for (int kb = 0; kb < nk; ++kb) {
          const int it = pass * nk + kb, st = it % ST;
          if (!mbar_wait(&full[st], (it / ST) & 1, abort_flag, err, 2)) {
            ok = false;
            break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          const uint32_t a0 = sptr(smem + st * kStage);
          const uint32_t b0 = a0 + S * kAplane;
          if (pass == 0) {
#pragma unroll
            for (int d = 0; d < D1; ++d)
#pragma unroll
              for (int p = 0; p <= d; ++p)
                mma_bf16(tmem + d * BN, sdesc_sw32(a0 + p * kAplane),
                         sdesc_sw32(b0 + (d - p) * kBplane), idesc, (kb > 0 || p > 0) ? 1u : 0u);
          } else {
#pragma unroll
            for (int d = D1; d < S; ++d)
#pragma unroll
              for (int p = 0; p <= d; ++p)
                mma_bf16(tmem + (d - D1) * BN, sdesc_sw32(a0 + p * kAplane),
                         sdesc_sw32(b0 + (d - p) * kBplane), idesc, (kb > 0 || p > 0) ? 1u : 0u);
          }
          mma_commit(&empty[st]);
        }
        mma_commit(&accf[pass]);
      }
      if (*abort_flag) {
        // the MMAs already issued must finish before TMEM is released
        uint64_t t0 = gtimer();
        while (!mbar_try(&accf[last], 0) && gtimer() - t0 < 1000000000ull) {
        }
      }
    }
  } else {
    const int q4 = warp & 3;
    const int m = m0 + q4 * 32 + lane;
    const int emr = (m < M) ? ea[z * Mpad + m] : 0;
    double* Cz = C + (size_t)z * strideC;
    for (int pass = 0; pass < 2; ++pass) {
      const bool ok = mbar_wait(&accf[pass], 0, abort_flag, err, 3, 1000);
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      if (!ok) break;
      const int d0 = pass ? D1 : 0, d1 = pass ? S : D1;
      for (int c0 = 0; c0 < BN; c0 += 16) {
        long long v[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) v[j] = 0;
        for (int d = d0; d < d1; ++d) {
          float f[16];
          tmem_ld16(tmem + ((uint32_t)(q4 * 32) << 16) + (d - d0) * BN + c0, f);
#pragma unroll
          for (int j = 0; j < 16; ++j) v[j] = (v[j] << w) + (long long)__float2int_rn(f[j]);
        }
        if (m < M) {
#pragma unroll
          for (int j = 0; j < 16; ++j) {
            const int n = n0 + c0 + j;
            if (n < Nc) {
              const int E = emr + eb[n] - 2 * w - w * (d1 - 1);
              double* dst = Cz + (size_t)n * ldc + m;
              const double part = scaled_int(v[j], E);
              *dst = (pass || accum) ? *dst + part : part;
            }
          }
        }
      }
      if (pass == 0) {
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(sptr(tfree)) : "memory");
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
  }
}


// Grouped-layout kernel.  TMA moves 32-byte rows at about a third of the rate
// of 128-byte rows into shared memory (16.7 vs 48.3 B/clk/SM measured on
// GB300), and the digit GEMM needs all s planes of a 16-wide K slice per
// stage.  In the grouped layout every 128-byte row holds that K slice for four
// planes (planes 4g..4g+3), so a stage is NQ = s/4 boxes of 128-byte rows plus
// NT = s%4 boxes of 32-byte rows per operand.  D1 = S runs the whole GEMM in
// one pass (all S accumulators in tensor memory, BN <= 512/S).
//
// Timeline of a tile (two passes): pass 0 (diagonals < D1) holds only D1
// planes per K slice, so when they fit twice a ring slot carries PK = 2 K
// slices and the MMA issuer stays ahead of the barrier round trip.  The eight
// epilogue warps (two per 32-lane TMEM quadrant, half the columns each) read
// all diagonals of a column chunk with one wait, fold them into exact int64
// sums, keep pass 0's sums in registers and release the tensor memory at once;
// pass 1's epilogue adds the two parts (one FP64 add per element) and stores.
constexpr int kThreadsG = 320;  // warp 0 TMA, warp 1 MMA, warps 2..9 epilogue
constexpr int kChunkG = 8;      // columns per tcgen05.ld in the epilogue

__device__ __forceinline__ void tmem_ld8_nowait(uint32_t taddr, uint32_t* r) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];\n"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
        "=r"(r[7])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait_ld() {
  asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
}

// ACC: add to C (the later launches of a K-segmented GEMM); a template
// argument, so the first launch's code carries no trace of it.
// PAIR: the tile is 256 x BN, computed by a cluster of two CTAs with
// tcgen05.mma.cta_group::2 (M = 256).  Each CTA loads its 128 rows of A and
// BN/2 rows of B; rank 0 waits for both CTAs' bytes on its own barriers (the
// rank-1 loads complete there), issues the MMAs and commits them to the
// barriers of both CTAs; both CTAs' epilogue warps read their own tensor
// memory (the tile's rows rank * 128 + lane, all BN columns).  Per SM, one
// MMA step reads 128 + BN/2 operand rows from shared memory instead of
// 128 + BN: the single-CTA kernel at BN = 96 is bound by that bandwidth.
constexpr int kStagesP = 4;
template <int S, int BN, int D1, bool ACC, bool KPARTS = false, bool PAIR = false>
__global__ void __launch_bounds__(kThreadsG, 1)
    k_split_gemm_g(const __grid_constant__ CUtensorMap tmAq, const __grid_constant__ CUtensorMap tmAt,
                   const __grid_constant__ CUtensorMap tmBq, const __grid_constant__ CUtensorMap tmBt,
                   const int32_t* __restrict__ ea, const int32_t* __restrict__ eb, double* C,
                   int ldc, size_t strideC, int M, int Mpad, int Nc, int K, int w, int nM, int nA,
                   int nN, int GA, int* err, int kpart_steps, size_t strideP) {
  constexpr int NQ = S / 4, NT = S % 4;
  constexpr int NPASS = D1 < S ? 2 : 1;
  constexpr int HALF = BN / 2;                     // columns per epilogue warp
  constexpr int NCH = HALF / kChunkG;              // chunks per epilogue warp
  constexpr int BNL = PAIR ? BN / 2 : BN;          // B rows this CTA loads
  static_assert(D1 * BN <= 512 && (S - D1) * BN <= 512, "tensor memory columns");
  static_assert((BNL * 128) % 1024 == 0, "128-byte-swizzle tiles stay 1024-byte aligned");
  static_assert(HALF % kChunkG == 0, "epilogue chunks");
  static_assert(!PAIR || (NPASS == 2 && !KPARTS && BN % 32 == 0), "pair: two-pass tiles");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t kAq = kBM * 128, kAt = kBM * 32, kBq = BNL * 128, kBt = BNL * 32;
  constexpr uint32_t kAbytes = NQ * kAq + NT * kAt;
  constexpr uint32_t kStage = stage_bytes_g(S, BNL);  // rounded up to 1024 bytes
  static_assert(kAbytes % 1024 == 0 && kStage >= kAbytes + NQ * kBq + NT * kBt, "stage layout");
  // pass 0 of a two-pass tile: D1 <= 4 planes are group 0 alone; two K slices
  // of it share a slot when they fit
  constexpr int PK = (NPASS == 2 && D1 <= 4 && 2 * (kAq + kBq) <= kStage) ? 2 : 1;
  constexpr int ST = PAIR ? kStagesP : kStages2;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST * kStage);
  uint64_t* empty = full + ST;
  uint64_t* accf = empty + ST;
  uint64_t* tfree = accf + 2;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(tfree + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);

  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const uint32_t rank = PAIR ? cluster_rank() : 0u;
  const int t = PAIR ? (int)(blockIdx.x >> 1) : (int)blockIdx.x;
  const int grp = t / (GA * nN);
  const int r = t - grp * GA * nN;
  const int gsz = min(GA, nA - grp * GA);
  const int ai = grp * GA + r % gsz;
  // a pair's tile has 256 rows (nM counts 256-row tiles); this CTA's are the
  // rank-th 128 of them
  const int n0 = (r / gsz) * BN, z = ai / nM;
  const int m0 = (ai % nM) * (PAIR ? 2 * kBM : kBM) + (int)rank * kBM;
  // K parts (grid y): part p contracts K steps [p * kpart_steps, ...) into its
  // own output C + p * strideP (kpart_steps = 0: one part, the whole K)
  const int kb0 = KPARTS ? (int)blockIdx.y * kpart_steps : 0;
  const int nk = KPARTS ? min(kpart_steps, K / kBK - kb0) : K / kBK;
  const int nk0 = nk / PK;  // ring slots of pass 0 (K parts are multiples of 64)
  const int nslots = nk0 + (NPASS == 2 ? nk : 0);

  if (threadIdx.x == 0) {
    for (int i = 0; i < ST; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&accf[0], 1);
    mbar_init(&accf[1], 1);
    mbar_init(tfree, PAIR ? 2 * 8 : 256);  // a pair: one arrival per epilogue warp of both CTAs
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    if constexpr (PAIR) {
      asm volatile("tcgen05.alloc.cta_group::2.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                       sptr(tmem_slot)));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::2.sync.aligned;\n");
    } else {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                       sptr(tmem_slot)));
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  // a pair: both CTAs' barriers are initialised before either signals the other's
  if constexpr (PAIR) cluster_sync_all();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;
  // rank 0's barrier of a slot, as a shared::cluster address (pairs)
  auto lead = [&](uint64_t* b) -> uint32_t { return PAIR ? mapa_shared(sptr(b), 0) : sptr(b); };

  if (warp == 0) {
    if (lane == 0) {  // TMA producer: both passes, one continuous slot ring
      int issued = 0;
      auto load = [&](void* dst, const CUtensorMap* map, int st, int c0, int c1, int c2) {
        if constexpr (PAIR) tma_load_3d_pair(dst, map, lead(&full[st]), c0, c1, c2);
        else tma_load_3d(dst, map, &full[st], c0, c1, c2);
      };
      // rank 0 expects the bytes of both CTAs (equal boxes); rank 1's loads
      // complete on rank 0's barrier, before or after that expectation
      auto expect = [&](int st, uint32_t bytes) {
        if (rank == 0) mbar_expect_tx(&full[st], PAIR ? 2 * bytes : bytes);
      };
      const int nb0 = n0 + (int)rank * BNL;  // this CTA's B rows
      for (int it = 0; it < nslots; ++it) {
        const int pass = it >= nk0, st = it % ST;
        if (it >= ST && !mbar_wait<PAIR>(&empty[st], ((it / ST) - 1) & 1, abort_flag, err, 21))
          break;
        unsigned char* sa = smem + st * kStage;
        if (pass == 0 && PK == 2) {
          expect(st, 2 * (kAq + kBq));
          for (int h = 0; h < 2; ++h) {
            const int kb = kb0 + 2 * it + h;
            unsigned char* sh = sa + h * (kAq + kBq);
            load(sh, &tmAq, st, kb * 64, z * Mpad + m0, 0);
            load(sh + kAq, &tmBq, st, kb * 64, nb0, 0);
          }
        } else {
          const int kb = kb0 + (pass ? it - nk0 : it);
          const int np = pass ? S : D1;
          const int gq = min(NQ, (np + 3) / 4), tq = max(0, np - 4 * NQ);
          unsigned char* sb = sa + kAbytes;
          expect(st, gq * (kAq + kBq) + tq * (kAt + kBt));
          for (int g = 0; g < gq; ++g) {
            load(sa + g * kAq, &tmAq, st, kb * 64, z * Mpad + m0, g);
            load(sb + g * kBq, &tmBq, st, kb * 64, nb0, g);
          }
          for (int q = 0; q < tq; ++q) {
            load(sa + NQ * kAq + q * kAt, &tmAt, st, kb * kBK, z * Mpad + m0, q);
            load(sb + NQ * kBq + q * kBt, &tmBt, st, kb * kBK, nb0, q);
          }
        }
        issued = it + 1;
      }
      if (*abort_flag) {
        if (rank == 0) {
          for (int it = (issued > ST ? issued - ST : 0); it < issued; ++it) {
            uint64_t t0 = gtimer();
            while (!(PAIR ? mbar_try_cl(&full[it % ST], (it / ST) & 1)
                          : mbar_try(&full[it % ST], (it / ST) & 1)) &&
                   gtimer() - t0 < 1000000000ull) {
            }
          }
        } else {
          // rank 1 cannot observe its loads (they complete on rank 0's
          // barriers): give them far longer than a load takes
          const uint64_t t0 = gtimer();
          while (gtimer() - t0 < 2000000ull) __nanosleep(1000);
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0 && rank == 0) {  // MMA issuer (rank 0 of a pair)
      const uint32_t idesc = idesc_bf16(PAIR ? 2 * kBM : kBM, BN);
      auto commit = [&](uint64_t* b) {
        if constexpr (PAIR) {
          mma_commit_pair(sptr(b));                   // this CTA's barrier
          mma_commit_pair(mapa_shared(sptr(b), 1));   // and rank 1's
        } else {
          mma_commit(b);
        }
      };
      auto mma = [&](uint32_t d, uint64_t a, uint64_t b, uint32_t idesc_, uint32_t acc) {
        if constexpr (PAIR) mma_bf16_pair(d, a, b, idesc_, acc);
        else mma_bf16(d, a, b, idesc_, acc);
      };
      bool ok = true;
      int last = 0;
      for (int it = 0; it < nslots && ok; ++it) {
        const int pass = it >= nk0, st = it % ST;
        if (pass == 1 && it == nk0) {  // pass 1 reuses pass 0's tensor memory
          commit(&accf[0]);
          last = 1;
          ok = mbar_wait<PAIR>(tfree, 0, abort_flag, err, 24);
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          if (!ok) break;
        }
        if (!mbar_wait<PAIR>(&full[st], (it / ST) & 1, abort_flag, err, 22)) {
          ok = false;
          break;
        }
        asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
        const uint32_t sa = sptr(smem + st * kStage);
        if (pass == 0 && PK == 2) {
#pragma unroll
          for (int h = 0; h < 2; ++h) {
            const uint32_t a0 = sa + h * (kAq + kBq), b0 = a0 + kAq;
            const bool first = it == 0 && h == 0;
#pragma unroll
            for (int d = 0; d < D1; ++d)
#pragma unroll
              for (int p = 0; p <= d; ++p)
                mma(tmem + d * BN, sdesc_sw128(a0 + p * 32), sdesc_sw128(b0 + (d - p) * 32),
                         idesc, (!first || p > 0) ? 1u : 0u);
          }
        } else {
          const uint32_t a0 = sa, b0 = sa + kAbytes;
          auto adesc = [&](int p) {
            return p < 4 * NQ ? sdesc_sw128(a0 + (p >> 2) * kAq + (p & 3) * 32)
                              : sdesc_sw32(a0 + NQ * kAq + (p - 4 * NQ) * kAt);
          };
          auto bdesc = [&](int p) {
            return p < 4 * NQ ? sdesc_sw128(b0 + (p >> 2) * kBq + (p & 3) * 32)
                              : sdesc_sw32(b0 + NQ * kBq + (p - 4 * NQ) * kBt);
          };
          const int kb = pass ? it - nk0 : it;
          if (pass == 0) {
#pragma unroll
            for (int d = 0; d < D1; ++d)
#pragma unroll
              for (int p = 0; p <= d; ++p)
                mma(tmem + d * BN, adesc(p), bdesc(d - p), idesc,
                         (kb > 0 || p > 0) ? 1u : 0u);
          } else {
#pragma unroll
            for (int d = D1; d < S; ++d)
#pragma unroll
              for (int p = 0; p <= d; ++p)
                mma(tmem + (d - D1) * BN, adesc(p), bdesc(d - p), idesc,
                         (kb > 0 || p > 0) ? 1u : 0u);
          }
        }
        commit(&empty[st]);
      }
      if (ok) commit(&accf[NPASS - 1]);
      if (*abort_flag) {
        uint64_t t0 = gtimer();
        while (!(PAIR ? mbar_try_cl(&accf[last], 0) : mbar_try(&accf[last], 0)) &&
               gtimer() - t0 < 1000000000ull) {
        }
      }
    }
  } else {
    // warps 2..9: TMEM lane quadrant (warp % 4), column half (warp - 2) / 4
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const int m = m0 + q4 * 32 + lane;
    const int emr = (m < M) ? ea[z * Mpad + m] : 0;
    double* Cz = C + (size_t)z * strideC + (KPARTS ? (size_t)blockIdx.y * strideP : 0);
    const uint32_t lanes = (uint32_t)(q4 * 32) << 16;
    long long v0[NCH][kChunkG];  // pass 0's exact sums of this thread's columns
    bool ok = true;
    for (int pass = 0; pass < NPASS && ok; ++pass) {
      ok = mbar_wait<PAIR>(&accf[pass], 0, abort_flag, err, 23, 256);
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      if (!ok) break;
      const int d0 = pass ? D1 : 0, d1 = pass ? S : D1;
#pragma unroll
      for (int ch = 0; ch < NCH; ++ch) {
        const int c0 = half * HALF + ch * kChunkG;
        // the earlier K segments' sums of this chunk, loaded before the
        // tensor-memory reads so that their latency overlaps them
        double prev[kChunkG];
        int ebc[kChunkG];  // the chunk's column exponents (last pass)
#pragma unroll
        for (int j = 0; j < kChunkG; ++j) {
          const int n = n0 + c0 + j;
          ebc[j] = (pass == NPASS - 1 && n < Nc) ? eb[n] : 0;
        }
        if constexpr (ACC) {
#pragma unroll
          for (int j = 0; j < kChunkG; ++j) {
            const int n = n0 + c0 + j;
            prev[j] = (pass == NPASS - 1 && m < M && n < Nc)
                          ? ld_acc(Cz + (size_t)n * ldc + m) : 0.0;
          }
        }
        uint32_t f[(D1 > S - D1 ? D1 : S - D1)][kChunkG];
#pragma unroll
        for (int d = 0; d < (D1 > S - D1 ? D1 : S - D1); ++d)
          if (d < d1 - d0) tmem_ld8_nowait(tmem + lanes + d * BN + c0, f[d]);
        tmem_wait_ld();
        // exact int64 sums: Horner in 2^w over at most SPLIT diagonals each
        // (a single pass keeps two of them, hi = d < SPLIT and lo = the rest,
        // so that no sum exceeds 2^63)
        constexpr int SPLIT = NPASS == 2 ? S : (S + 1) / 2;
        long long v[kChunkG], hi[kChunkG];
#pragma unroll
        for (int j = 0; j < kChunkG; ++j) v[j] = hi[j] = 0;
#pragma unroll
        for (int d = 0; d < (D1 > S - D1 ? D1 : S - D1); ++d)
          if (d < d1 - d0) {
            if (NPASS == 1 && d == SPLIT) {
#pragma unroll
              for (int j = 0; j < kChunkG; ++j) {
                hi[j] = v[j];
                v[j] = 0;
              }
            }
#pragma unroll
            for (int j = 0; j < kChunkG; ++j)
              v[j] = (v[j] << w) + (long long)__float2int_rn(__uint_as_float(f[d][j]));
          }
        if (pass == 0 && NPASS == 2) {
#pragma unroll
          for (int j = 0; j < kChunkG; ++j) v0[ch][j] = v[j];
        } else if (m < M) {
          double outc[kChunkG];
#pragma unroll
          for (int j = 0; j < kChunkG; j += 2) {
            const int b0 = emr + ebc[j] - 2 * w, b1 = emr + ebc[j + 1] - 2 * w;
            const double2 o =
                NPASS == 2
                    ? scaled_pair2(v0[ch][j], b0 - w * (D1 - 1), v[j], b0 - w * (d1 - 1),
                                   v0[ch][j + 1], b1 - w * (D1 - 1), v[j + 1], b1 - w * (d1 - 1))
                    : scaled_pair2(hi[j], b0 - w * (SPLIT - 1), v[j], b0 - w * (d1 - 1),
                                   hi[j + 1], b1 - w * (SPLIT - 1), v[j + 1], b1 - w * (d1 - 1));
            outc[j] = o.x;
            outc[j + 1] = o.y;
          }
#pragma unroll
          for (int j = 0; j < kChunkG; ++j) {
            const int n = n0 + c0 + j;
            if (n < Nc) {
              double out = outc[j];
              double* dst = Cz + (size_t)n * ldc + m;
              if constexpr (ACC) out += prev[j];
              *dst = out;
            }
          }
        }
      }
      if (pass == 0 && NPASS == 2) {  // all reads done: pass 1 may overwrite the columns
        asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
        if constexpr (PAIR) {  // one arrival per warp, on rank 0's barrier
          __syncwarp();
          if (lane == 0) mbar_arrive_cl(lead(tfree));
        } else {
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(sptr(tfree)) : "memory");
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  // a pair: neither CTA frees its tensor memory or exits (its shared memory
  // and barriers) while the other may still address them
  if constexpr (PAIR) cluster_sync_all();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    if constexpr (PAIR)
      asm volatile("tcgen05.dealloc.cta_group::2.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
    else
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
  }
}

// ------------------------------------------------------------------ grouped persistent
// Persistent multi-problem form of the two-pass grouped kernel (one launch for
// the final-state GEMMs of every final block of a round).  The problems (one
// per final block: its vectors' digits x its H digits) have their own shapes
// and K; their tiles form one work list, problem by problem, row tiles
// fastest.  One CTA per SM takes items blockIdx.x, blockIdx.x + gridDim.x, ...
// and runs each item's K in segments of at most kKSeg (the exactness bound of
// the diagonal sums), each segment's FP64 result added to the previous ones'
// by the same epilogue thread.  Tensor memory holds one segment at a time, so
// the barriers that hand it between the MMA issuer and the epilogue count
// segments: accf[p] completes once per segment and pass, tfree0 / tfree1 once
// per segment after the epilogue has read pass 0 / pass 1.
constexpr int kGpMaxProb = 44;  // 44 x 640 B of kernel parameters (limit 32,764 B)

struct GpProb {
  CUtensorMap aq, at, bq, bt;
  const int32_t* ea;
  const int32_t* eb;
  double* C;
  int ldc, M, Mpad, Nc, K, nM, nN, first;  // first: the problem's first work item
  // the fused epilogue: the block's parts (initial units, sorted by column)
  // and its final levels' energies, upper-filter flags and line ids
  const EpiPart* parts;
  const double* EF;
  const uint8_t* upper;
  const int32_t* lvF;
  int nparts;
};
static_assert(sizeof(GpProb) <= 640, "problem parameters");
struct GpParams {
  GpProb p[kGpMaxProb];
  int nprob, nitems;
  // fused: the last K segment's epilogue forms the lines (epilogue.cuh)
  // instead of storing T
  int fused;
  gi_line* out;
  unsigned long long* counter;
  long long cap;
  RefineRec* rec;
  long long rec_cap;
};
static_assert(sizeof(GpParams) <= 32764, "kernel parameter limit");

// The fused epilogue of one 8-column chunk of a final block's T, held by one
// thread for final level f = m: groups of G consecutive columns are the
// moments of one initial level (G = ndegI * ndegF combinations).
template <int G>
__device__ __forceinline__ void fused_chunk(const GpParams& P, const GpProb& pr, int nbase, int m,
                                            bool row_ok, const double* outv) {
#pragma unroll
  for (int g0 = 0; g0 < kChunkG; g0 += G) {
    const int n = nbase + g0;
    if (n >= pr.Nc) break;  // the same for every lane of the warp
    int q = 0;
    while (q + 1 < pr.nparts && pr.parts[q + 1].c0 <= n) ++q;
    const EpiPart& pt = pr.parts[q];
    const EpiParams& ep = pt.ep;
    const int i = (n - pt.c0) / G;
    // column offset dI * ndegF + dF within the group -> moment index dI + 2 dF
    double t[4] = {0.0, 0.0, 0.0, 0.0}, hnq[4] = {0.0, 0.0, 0.0, 0.0};
#pragma unroll
    for (int o = 0; o < G; ++o) {
      const int dI = (G == 4) ? (o >> 1) : (G == 2 ? (ep.ndegF == 1 ? o : 0) : 0);
      const int dF = (G == 4) ? (o & 1) : (G == 2 ? (ep.ndegF == 1 ? 0 : o) : 0);
      if (ep.combo_mask & (1 << (dI + 2 * dF))) {
        t[dI + 2 * dF] = outv[g0 + o];
        hnq[dI + 2 * dF] = pt.hn[i * G + o];
      }
    }
    const bool ok_f = row_ok && pr.upper[m];
    LineEval r;
    eval_line(ep, t, hnq, pt.EI[i], ok_f ? pr.EF[m] : 0.0, pt.BI[i], ok_f, pt.lvI[i],
              ok_f ? pr.lvF[m] : -1, r);
    append_line(r, ep.part, i, m, P.out, P.counter, P.cap, P.rec, P.rec_cap);
  }
}

template <int S, int BN, int D1>
__global__ void __launch_bounds__(kThreadsG, 1)
    k_split_gemm_gp(const __grid_constant__ GpParams P, int w, int* err) {
  constexpr int NQ = S / 4, NT = S % 4;
  constexpr int HALF = BN / 2, NCH = HALF / kChunkG;
  constexpr int MAXD = D1 > S - D1 ? D1 : S - D1;
  static_assert(D1 < S && D1 * BN <= 512 && (S - D1) * BN <= 512, "tensor memory columns");
  static_assert((BN * 128) % 1024 == 0 && HALF % kChunkG == 0, "tile shape");
  extern __shared__ __align__(1024) unsigned char smem_raw[];
  unsigned char* smem = reinterpret_cast<unsigned char*>(
      (reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  constexpr uint32_t kAq = kBM * 128, kAt = kBM * 32, kBq = BN * 128, kBt = BN * 32;
  constexpr uint32_t kAbytes = NQ * kAq + NT * kAt;
  constexpr uint32_t kStage = stage_bytes_g(S, BN);
  constexpr int PK = (D1 <= 4 && 2 * (kAq + kBq) <= kStage) ? 2 : 1;
  constexpr int ST = kStages2;
  uint64_t* full = reinterpret_cast<uint64_t*>(smem + ST * kStage);
  uint64_t* empty = full + ST;
  uint64_t* accf = empty + ST;    // [2]
  uint64_t* tfree0 = accf + 2;
  uint64_t* tfree1 = tfree0 + 1;
  uint64_t* drain = tfree1 + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(drain + 1);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(tmem_slot + 1);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;

  if (threadIdx.x == 0) {
    for (int i = 0; i < ST; ++i) {
      mbar_init(&full[i], 1);
      mbar_init(&empty[i], 1);
    }
    mbar_init(&accf[0], 1);
    mbar_init(&accf[1], 1);
    mbar_init(tfree0, 256);
    mbar_init(tfree1, 256);
    mbar_init(drain, 1);
    *abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;\n" ::"r"(
                     sptr(tmem_slot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = *tmem_slot;

  // item -> (problem, row tile, column tile); every role walks the same list
  auto decode = [&](int item, int& pi, int& m0, int& n0) {
    pi = 0;
    while (pi + 1 < P.nprob && P.p[pi + 1].first <= item) ++pi;
    const int local = item - P.p[pi].first;
    m0 = (local % P.p[pi].nM) * kBM;
    n0 = (local / P.p[pi].nM) * BN;
  };

  if (warp == 0) {
    if (lane == 0) {  // TMA producer: one continuous slot ring over all segments
      int it = 0;
      bool ok = true;
      for (int item = blockIdx.x; item < P.nitems && ok; item += gridDim.x) {
        int pi, m0, n0;
        decode(item, pi, m0, n0);
        const GpProb& pr = P.p[pi];
        for (int k0 = 0; k0 < pr.K && ok; k0 += kKSeg) {
          const int nk = min(kKSeg, pr.K - k0) / kBK, nk0 = nk / PK;
          for (int sl = 0; sl < nk0 + nk; ++sl, ++it) {
            const int pass = sl >= nk0, st = it % ST;
            if (it >= ST && !mbar_wait(&empty[st], ((it / ST) - 1) & 1, abort_flag, err, 31)) {
              ok = false;
              break;
            }
            unsigned char* sa = smem + st * kStage;
            if (pass == 0 && PK == 2) {
              mbar_expect_tx(&full[st], 2 * (kAq + kBq));
              for (int h = 0; h < 2; ++h) {
                const int kb = k0 / kBK + 2 * sl + h;
                unsigned char* sh = sa + h * (kAq + kBq);
                tma_load_3d(sh, &pr.aq, &full[st], kb * 64, m0, 0);
                tma_load_3d(sh + kAq, &pr.bq, &full[st], kb * 64, n0, 0);
              }
            } else {
              const int kb = k0 / kBK + (pass ? sl - nk0 : sl);
              const int np = pass ? S : D1;
              const int gq = min(NQ, (np + 3) / 4), tq = max(0, np - 4 * NQ);
              unsigned char* sb = sa + kAbytes;
              mbar_expect_tx(&full[st], gq * (kAq + kBq) + tq * (kAt + kBt));
              for (int g = 0; g < gq; ++g) {
                tma_load_3d(sa + g * kAq, &pr.aq, &full[st], kb * 64, m0, g);
                tma_load_3d(sb + g * kBq, &pr.bq, &full[st], kb * 64, n0, g);
              }
              for (int q = 0; q < tq; ++q) {
                tma_load_3d(sa + NQ * kAq + q * kAt, &pr.at, &full[st], kb * kBK, m0, q);
                tma_load_3d(sb + NQ * kBq + q * kBt, &pr.bt, &full[st], kb * kBK, n0, q);
              }
            }
          }
        }
      }
      if (*abort_flag) {  // copies in flight land before the shared memory goes away
        for (int j = (it > ST ? it - ST : 0); j < it; ++j) {
          const uint64_t t0 = gtimer();
          while (!mbar_try(&full[j % ST], (j / ST) & 1) && gtimer() - t0 < 1000000000ull) {
          }
        }
      }
    }
  } else if (warp == 1) {
    if (lane == 0) {  // MMA issuer
      const uint32_t idesc = idesc_bf16(kBM, BN);
      int it = 0, seg = 0;  // ring slot and segment counters of this CTA
      bool ok = true;
      for (int item = blockIdx.x; item < P.nitems && ok; item += gridDim.x) {
        int pi, m0, n0;
        decode(item, pi, m0, n0);
        const int K = P.p[pi].K;
        for (int k0 = 0; k0 < K && ok; k0 += kKSeg, ++seg) {
          const int nk = min(kKSeg, K - k0) / kBK, nk0 = nk / PK;
          if (seg > 0) {  // the epilogue has read the previous segment's pass 1
            ok = mbar_wait(tfree1, (seg - 1) & 1, abort_flag, err, 34);
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            if (!ok) break;
          }
          for (int sl = 0; sl < nk0 + nk; ++sl, ++it) {
            const int pass = sl >= nk0, st = it % ST;
            if (pass == 1 && sl == nk0) {  // pass 1 reuses pass 0's tensor memory
              mma_commit(&accf[0]);
              ok = mbar_wait(tfree0, seg & 1, abort_flag, err, 35);
              asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
              if (!ok) break;
            }
            if (!mbar_wait(&full[st], (it / ST) & 1, abort_flag, err, 32)) {
              ok = false;
              break;
            }
            asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
            const uint32_t sa = sptr(smem + st * kStage);
            if (pass == 0 && PK == 2) {
#pragma unroll
              for (int h = 0; h < 2; ++h) {
                const uint32_t a0 = sa + h * (kAq + kBq), b0 = a0 + kAq;
                const bool first = sl == 0 && h == 0;
#pragma unroll
                for (int d = 0; d < D1; ++d)
#pragma unroll
                  for (int p = 0; p <= d; ++p)
                    mma_bf16(tmem + d * BN, sdesc_sw128(a0 + p * 32),
                             sdesc_sw128(b0 + (d - p) * 32), idesc, (!first || p > 0) ? 1u : 0u);
              }
            } else {
              const uint32_t a0 = sa, b0 = sa + kAbytes;
              auto adesc = [&](int p) {
                return p < 4 * NQ ? sdesc_sw128(a0 + (p >> 2) * kAq + (p & 3) * 32)
                                  : sdesc_sw32(a0 + NQ * kAq + (p - 4 * NQ) * kAt);
              };
              auto bdesc = [&](int p) {
                return p < 4 * NQ ? sdesc_sw128(b0 + (p >> 2) * kBq + (p & 3) * 32)
                                  : sdesc_sw32(b0 + NQ * kBq + (p - 4 * NQ) * kBt);
              };
              const int kb = pass ? sl - nk0 : sl;
              if (pass == 0) {
#pragma unroll
                for (int d = 0; d < D1; ++d)
#pragma unroll
                  for (int p = 0; p <= d; ++p)
                    mma_bf16(tmem + d * BN, adesc(p), bdesc(d - p), idesc,
                             (kb > 0 || p > 0) ? 1u : 0u);
              } else {
#pragma unroll
                for (int d = D1; d < S; ++d)
#pragma unroll
                  for (int p = 0; p <= d; ++p)
                    mma_bf16(tmem + (d - D1) * BN, adesc(p), bdesc(d - p), idesc,
                             (kb > 0 || p > 0) ? 1u : 0u);
              }
            }
            mma_commit(&empty[st]);
          }
          if (ok) mma_commit(&accf[1]);
        }
      }
      // every MMA issued has completed before the tensor memory is freed
      mma_commit(drain);
      const uint64_t t0 = gtimer();
      while (!mbar_try(drain, 0) && gtimer() - t0 < 1000000000ull) {
      }
    }
  } else {
    // warps 2..9: TMEM lane quadrant (warp % 4), column half (warp - 2) / 4
    const int q4 = warp & 3, half = (warp - 2) >> 2;
    const uint32_t lanes = (uint32_t)(q4 * 32) << 16;
    int seg = 0;
    bool ok = true;
    for (int item = blockIdx.x; item < P.nitems && ok; item += gridDim.x) {
      int pi, m0, n0;
      decode(item, pi, m0, n0);
      const GpProb& pr = P.p[pi];
      const int m = m0 + q4 * 32 + lane;
      const int emr = (m < pr.M) ? pr.ea[m] : 0;
      for (int k0 = 0; k0 < pr.K && ok; k0 += kKSeg, ++seg) {
        long long v0[NCH][kChunkG];  // pass 0's exact sums of this thread's columns
        for (int pass = 0; pass < 2 && ok; ++pass) {
          ok = mbar_wait(&accf[pass], seg & 1, abort_flag, err, 33, 256);
          asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
          if (!ok) break;
          const int d0 = pass ? D1 : 0, d1 = pass ? S : D1;
#pragma unroll
          for (int ch = 0; ch < NCH; ++ch) {
            const int c0 = half * HALF + ch * kChunkG;
            // the earlier segments' sums of this chunk, loaded before the
            // tensor-memory reads so that their latency overlaps them
            double prev[kChunkG];
            int ebc[kChunkG];  // the chunk's column exponents (pass 1)
#pragma unroll
            for (int j = 0; j < kChunkG; ++j) {
              const int n = n0 + c0 + j;
              ebc[j] = (pass == 1 && n < pr.Nc) ? pr.eb[n] : 0;
            }
#pragma unroll
            for (int j = 0; j < kChunkG; ++j) {
              const int n = n0 + c0 + j;
              prev[j] = (pass == 1 && k0 > 0 && m < pr.M && n < pr.Nc)
                            ? ld_acc(pr.C + (size_t)n * pr.ldc + m) : 0.0;
            }
            uint32_t f[MAXD][kChunkG];
#pragma unroll
            for (int d = 0; d < MAXD; ++d)
              if (d < d1 - d0) tmem_ld8_nowait(tmem + lanes + d * BN + c0, f[d]);
            tmem_wait_ld();
            long long v[kChunkG];
#pragma unroll
            for (int j = 0; j < kChunkG; ++j) v[j] = 0;
#pragma unroll
            for (int d = 0; d < MAXD; ++d)
              if (d < d1 - d0) {
#pragma unroll
                for (int j = 0; j < kChunkG; ++j)
                  v[j] = (v[j] << w) + (long long)__float2int_rn(__uint_as_float(f[d][j]));
              }
            if (pass == 0) {
#pragma unroll
              for (int j = 0; j < kChunkG; ++j) v0[ch][j] = v[j];
            } else {
              // the last segment of a fused launch forms the lines; every
              // other segment stores its sum for the next one
              const bool row_ok = m < pr.M;
              const bool lines = P.fused && k0 + kKSeg >= pr.K;
              double outc[kChunkG], outv[kChunkG];
#pragma unroll
              for (int j = 0; j < kChunkG; j += 2) {
                const int b0 = emr + ebc[j] - 2 * w, b1 = emr + ebc[j + 1] - 2 * w;
                const double2 o = scaled_pair2(v0[ch][j], b0 - w * (D1 - 1), v[j],
                                               b0 - w * (S - 1), v0[ch][j + 1],
                                               b1 - w * (D1 - 1), v[j + 1], b1 - w * (S - 1));
                outc[j] = o.x;
                outc[j + 1] = o.y;
              }
#pragma unroll
              for (int j = 0; j < kChunkG; ++j) {
                const int n = n0 + c0 + j;
                outv[j] = 0.0;
                if (row_ok && n < pr.Nc) {
                  double out = outc[j];
                  double* dst = pr.C + (size_t)n * pr.ldc + m;
                  if (k0 > 0) out += prev[j];  // the earlier segments' sum
                  if (!lines) *dst = out;
                  outv[j] = out;
                }
              }
              if (lines) {
                const int G = pr.parts[0].grp;
                if (G == 4)
                  fused_chunk<4>(P, pr, n0 + c0, m, row_ok, outv);
                else if (G == 2)
                  fused_chunk<2>(P, pr, n0 + c0, m, row_ok, outv);
                else
                  fused_chunk<1>(P, pr, n0 + c0, m, row_ok, outv);
              }
            }
          }
          // all reads of this pass are done: the MMA issuer may overwrite the columns
          asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
          asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];\n" ::"r"(
                           sptr(pass ? tfree1 : tfree0))
                       : "memory");
        }
      }
    }
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 1) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;\n" ::"r"(tmem));
  }
}

// ------------------------------------------------------------------ slicing
// FP64 arithmetic is scarce on this GPU, so the digits are cut with integer
// operations on the bit pattern.  For a row with exponent e (max|x| < 2^(e-1)),
// each element becomes the fixed-point integer X = round(x 2^(ws - e)),
// |X| <= 2^(ws-1), and X is split from the bottom into balanced base-2^w
// digits: a_p in [-2^(w-1), 2^(w-1)) for p >= 1 and the remaining top digit
// |a_0| <= 2^(w-1), so X = sum_p a_p 2^(w(s-1-p)) exactly.

// Row exponent from the largest magnitude's bit pattern: 2^(e-1) <= max < 2^e.
__device__ __forceinline__ int row_exponent(unsigned long long maxbits) {
  if (maxbits == 0) return 0;
  const int eb = (int)(maxbits >> 52);
  return eb ? eb - 1022 : -1021 - (__clzll((long long)maxbits) - 12);
}

__device__ __forceinline__ long long fixed_point(double x, int e, int ws) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(x);
  const int eb = (int)((b >> 52) & 0x7FF);
  const long long mant = (long long)(b & 0xFFFFFFFFFFFFFull) | (eb ? (1ll << 52) : 0ll);
  const int sh = (eb ? eb : 1) - 1075 - e + ws;  // x 2^(ws-e) = mant 2^sh
  long long X;
  if (sh >= 0) {
    X = mant << sh;
  } else if (sh > -54) {
    X = (mant + (1ll << (-sh - 1))) >> (-sh);  // round half up
  } else {
    X = 0;
  }
  return (b >> 63) ? -X : X;
}

__device__ __forceinline__ uint16_t bf16_of_int(int a) {
  const __nv_bfloat16 h = __float2bfloat16_rn((float)a);  // |a| <= 256: exact
  return *reinterpret_cast<const uint16_t*>(&h);
}

// One warp per row, two elements per lane: out[p][r][k] (plane-major) and the
// row exponent.  Rows beyond `rows` are zero; K is even.  blockIdx.y selects
// one of gridDim.y stacked operands (X + y * xstride), whose rows go to rows
// [y * rows_pad, (y + 1) * rows_pad) of a plane set of gridDim.y * rows_pad rows.
// Element offset of digit (plane p, row r, element k) in a [s][rows][K] plane
// set: plain, or grouped (planes 4g..4g+3 interleaved per 16-element K slice in
// one 4K-wide row, the s % 4 remaining planes plain after them).
__host__ __device__ __forceinline__ size_t digit_offset(bool grouped, int s, int p, size_t r,
                                                        int k, int K, size_t rows) {
  const int nq = grouped ? s / 4 : 0;
  if (p < 4 * nq)
    return ((size_t)(p >> 2) * rows + r) * 4 * (size_t)K + (size_t)(k >> 4) * 64 + (p & 3) * 16 +
           (k & 15);
  return (size_t)4 * nq * rows * K + ((size_t)(p - 4 * nq) * rows + r) * K + k;
}

__global__ void k_slice_rows(const double* __restrict__ X, int ldx, size_t xstride, int rows,
                             int K, int rows_pad, int s, int w, uint32_t* __restrict__ out,
                             int grouped, int32_t* __restrict__ e_out) {
  const int r = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (r >= rows_pad) return;
  const size_t rset = (size_t)gridDim.y * rows_pad;         // rows of the plane set
  const size_t ro = (size_t)blockIdx.y * rows_pad + r;      // this row in the set
  const double2* x2 =
      reinterpret_cast<const double2*>(X + blockIdx.y * xstride + (size_t)r * ldx);
  const int K2 = K >> 1;
  unsigned long long mx = 0;
  if (r < rows)
    for (int k = lane; k < K2; k += 32) {
      const double2 v = x2[k];
      mx = max(mx, (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull);
      mx = max(mx, (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull);
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  const int e = row_exponent(mx) + 1;  // |x| < 2^(e-1): every digit within 2^(w-1)
  if (lane == 0) e_out[ro] = e;
  const int ws = w * s;
  const long long half = 1ll << (w - 1), mask = (1ll << w) - 1;
  for (int k = lane; k < K2; k += 32) {
    long long X0 = 0, X1 = 0;
    if (r < rows) {
      const double2 v = x2[k];
      X0 = fixed_point(v.x, e, ws);
      X1 = fixed_point(v.y, e, ws);
    }
    // elements 2k and 2k+1 are adjacent in both layouts: one 32-bit store
    for (int p = s - 1; p >= 1; --p) {
      const long long a0 = ((X0 + half) & mask) - half;
      const long long a1 = ((X1 + half) & mask) - half;
      X0 = (X0 - a0) >> w;
      X1 = (X1 - a1) >> w;
      out[digit_offset(grouped, s, p, ro, 2 * k, K, rset) >> 1] =
          (uint32_t)bf16_of_int((int)a0) | ((uint32_t)bf16_of_int((int)a1) << 16);
    }
    out[digit_offset(grouped, s, 0, ro, 2 * k, K, rset) >> 1] =
        (uint32_t)bf16_of_int((int)X0) | ((uint32_t)bf16_of_int((int)X1) << 16);
  }
}

// The same cut with one 256-thread block per row and the digit count fixed at
// compile time (the planes' row bases in registers, the digit loop unrolled):
// rows as long as a final block's basis (~11k elements) keep enough loads in
// flight, where one warp per row leaves the kernel latency-bound.
// One row of k_slice_rows_b: row ro of a plane set of rset rows, x2 its K
// values (valid: a row of X, else zeros).
template <int S>
__device__ __forceinline__ void slice_row_b(const double2* __restrict__ x2, bool valid, int K,
                                            int w, uint32_t* __restrict__ out, int grouped,
                                            int32_t* __restrict__ e_out, size_t ro, size_t rset) {
  __shared__ unsigned long long wmax[8];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int K2 = K >> 1;
  unsigned long long mx = 0;
  if (valid)
    for (int k = threadIdx.x; k < K2; k += 256) {
      const double2 v = x2[k];
      mx = max(mx, (unsigned long long)__double_as_longlong(v.x) & 0x7FFFFFFFFFFFFFFFull);
      mx = max(mx, (unsigned long long)__double_as_longlong(v.y) & 0x7FFFFFFFFFFFFFFFull);
    }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) wmax[warp] = mx;
  __syncthreads();
  mx = wmax[0];
#pragma unroll
  for (int i = 1; i < 8; ++i) mx = max(mx, wmax[i]);
  const int e = row_exponent(mx) + 1;  // |x| < 2^(e-1): every digit within 2^(w-1)
  if (threadIdx.x == 0) e_out[ro] = e;
  // 32-bit word offsets: plane p of this row starts at base[p]; the pair of
  // elements (2k, 2k+1) lies koff words further (digit_offset's layouts)
  const int nq = grouped ? S / 4 : 0;
  size_t base[S];
#pragma unroll
  for (int p = 0; p < S; ++p)
    base[p] = p < 4 * nq ? (((size_t)(p >> 2) * rset + ro) * 4 * (size_t)K + (p & 3) * 16) >> 1
                         : ((size_t)4 * nq * rset * K + ((size_t)(p - 4 * nq) * rset + ro) * K) >> 1;
  const int ws = w * S;
  const long long half = 1ll << (w - 1), mask = (1ll << w) - 1;
  for (int k = threadIdx.x; k < K2; k += 256) {
    long long X0 = 0, X1 = 0;
    if (valid) {
      const double2 v = x2[k];
      X0 = fixed_point(v.x, e, ws);
      X1 = fixed_point(v.y, e, ws);
    }
    const size_t kg = (size_t)(k >> 3) * 32 + (k & 7);
#pragma unroll
    for (int p = S - 1; p >= 1; --p) {
      const long long a0 = ((X0 + half) & mask) - half;
      const long long a1 = ((X1 + half) & mask) - half;
      X0 = (X0 - a0) >> w;
      X1 = (X1 - a1) >> w;
      out[base[p] + (p < 4 * nq ? kg : (size_t)k)] =
          (uint32_t)bf16_of_int((int)a0) | ((uint32_t)bf16_of_int((int)a1) << 16);
    }
    out[base[0] + (4 * nq > 0 ? kg : (size_t)k)] =
        (uint32_t)bf16_of_int((int)X0) | ((uint32_t)bf16_of_int((int)X1) << 16);
  }
}

template <int S>
__global__ void __launch_bounds__(256) k_slice_rows_b(const double* __restrict__ X, int ldx,
                                                      size_t xstride, int rows, int K,
                                                      int rows_pad, int w,
                                                      uint32_t* __restrict__ out, int grouped,
                                                      int32_t* __restrict__ e_out) {
  const int r = blockIdx.x;
  const size_t rset = (size_t)gridDim.y * rows_pad;     // rows of the plane set
  const size_t ro = (size_t)blockIdx.y * rows_pad + r;  // this row in the set
  const double2* x2 =
      reinterpret_cast<const double2*>(X + blockIdx.y * xstride + (size_t)r * ldx);
  slice_row_b<S>(x2, r < rows, K, w, out, grouped, e_out, ro, rset);
}

// The rows of several operands in one launch (each its own plane set, every
// row valid): operand j has rows [row0[j], row0[j + 1]) of the grid.
constexpr int kSliceMaxOps = 44;
struct SliceOps {
  int n;
  int row0[kSliceMaxOps + 1];
  int K[kSliceMaxOps];
  int ldx[kSliceMaxOps];
  const double* X[kSliceMaxOps];
  uint32_t* out[kSliceMaxOps];
  int32_t* e[kSliceMaxOps];
};
template <int S>
__global__ void __launch_bounds__(256) k_slice_rows_ops(const __grid_constant__ SliceOps ops,
                                                        int w, int grouped) {
  const int b = blockIdx.x;
  int j = 0;
  while (j + 1 < ops.n && ops.row0[j + 1] <= b) ++j;
  const int r = b - ops.row0[j];
  const size_t rows = (size_t)(ops.row0[j + 1] - ops.row0[j]);
  const double2* x2 = reinterpret_cast<const double2*>(ops.X[j] + (size_t)r * ops.ldx[j]);
  slice_row_b<S>(x2, true, ops.K[j], w, ops.out[j], grouped, ops.e[j], (size_t)r, rows);
}

// Y built straight into its digit planes (split path): one 256-thread block per
// row (i, d, slot) of the B operand computes the row's Kp values of Y with
// k_build_y's arithmetic (the same order of operations, so the same doubles)
// into shared memory, takes the row exponent and cuts the digits as
// k_slice_rows_b does.  The FP64 Y never goes to HBM.
// One row of Y (row = (i * ndeg + d) * nslot + slot within the unit) into its
// digit planes: the row in shared memory, its exponent, its digits.
template <int S>
__device__ __forceinline__ void build_y_digits_row(
    const double* __restrict__ vecs, int ld, const int32_t* __restrict__ ivec, int ndeg,
    const int32_t* __restrict__ yptr, const int32_t* __restrict__ yroot,
    const int32_t* __restrict__ root_case, const int32_t* __restrict__ root_lam,
    const int32_t* __restrict__ case_iterm, const int32_t* __restrict__ case_nelem,
    const double* __restrict__ rep, int Ntot, int degen, int nslot, int N, int Kp, int w,
    uint32_t* __restrict__ out, int grouped, int32_t* __restrict__ e_out, size_t row0,
    size_t rset, int row) {
  extern __shared__ __align__(16) double ys[];  // the row's Kp values
  __shared__ unsigned long long wmax[8];
  const int col = row / nslot, slot = row - col * nslot;
  const int i = col / ndeg, d = col - i * ndeg;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const double* vs = vecs + (size_t)ivec[i] * ld;
  const double* rd = rep + (size_t)d * Ntot;
  unsigned long long mx = 0;
  for (int v = threadIdx.x; v < Kp; v += 256) {
    double acc = 0.0;
    if (v < N) {
      const int q = slot * N + v;
      for (int p = yptr[q]; p < yptr[q + 1]; ++p) {
        const int r = yroot[p];
        const int c = root_case[r], lam = root_lam[r];
        const int it = case_iterm[c], ne = case_nelem[c];
        const double* rr = rd + (size_t)lam * degen * Ntot;
        for (int j = 0; j < ne; ++j) acc = fma(vs[it + j], rr[it + j], acc);
      }
    }
    ys[v] = acc;
    mx = max(mx, (unsigned long long)__double_as_longlong(acc) & 0x7FFFFFFFFFFFFFFFull);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) mx = max(mx, __shfl_xor_sync(0xffffffffu, mx, o));
  if (lane == 0) wmax[warp] = mx;
  __syncthreads();  // also: every value of the row is in shared memory
  mx = wmax[0];
#pragma unroll
  for (int q = 1; q < 8; ++q) mx = max(mx, wmax[q]);
  const int e = row_exponent(mx) + 1;
  const size_t ro = row0 + row;
  if (threadIdx.x == 0) e_out[ro] = e;
  const int nq = grouped ? S / 4 : 0;
  size_t base[S];
#pragma unroll
  for (int p = 0; p < S; ++p)
    base[p] = p < 4 * nq ? (((size_t)(p >> 2) * rset + ro) * 4 * (size_t)Kp + (p & 3) * 16) >> 1
                         : ((size_t)4 * nq * rset * Kp + ((size_t)(p - 4 * nq) * rset + ro) * Kp) >> 1;
  const int ws = w * S;
  const long long half = 1ll << (w - 1), mask = (1ll << w) - 1;
  const double2* y2 = reinterpret_cast<const double2*>(ys);
  for (int k = threadIdx.x; k < (Kp >> 1); k += 256) {
    const double2 v = y2[k];
    long long X0 = fixed_point(v.x, e, ws), X1 = fixed_point(v.y, e, ws);
    const size_t kg = (size_t)(k >> 3) * 32 + (k & 7);
    if ((X0 | X1) == 0) {  // most of Y is zero: every digit of the pair is zero
#pragma unroll
      for (int p = 0; p < S; ++p) out[base[p] + (p < 4 * nq ? kg : (size_t)k)] = 0u;
      continue;
    }
#pragma unroll
    for (int p = S - 1; p >= 1; --p) {
      const long long a0 = ((X0 + half) & mask) - half;
      const long long a1 = ((X1 + half) & mask) - half;
      X0 = (X0 - a0) >> w;
      X1 = (X1 - a1) >> w;
      out[base[p] + (p < 4 * nq ? kg : (size_t)k)] =
          (uint32_t)bf16_of_int((int)a0) | ((uint32_t)bf16_of_int((int)a1) << 16);
    }
    out[base[0] + (4 * nq > 0 ? kg : (size_t)k)] =
        (uint32_t)bf16_of_int((int)X0) | ((uint32_t)bf16_of_int((int)X1) << 16);
  }}

template <int S>
__global__ void __launch_bounds__(256)
    k_build_y_digits(const double* __restrict__ vecs, int ld, const int32_t* __restrict__ ivec,
                     int ndeg, const int32_t* __restrict__ yptr, const int32_t* __restrict__ yroot,
                     const int32_t* __restrict__ root_case, const int32_t* __restrict__ root_lam,
                     const int32_t* __restrict__ case_iterm,
                     const int32_t* __restrict__ case_nelem, const double* __restrict__ rep,
                     int Ntot, int degen, int nslot, int N, int Kp, int w,
                     uint32_t* __restrict__ out, int grouped, int32_t* __restrict__ e_out,
                     size_t row0, size_t rset) {
  build_y_digits_row<S>(vecs, ld, ivec, ndeg, yptr, yroot, root_case, root_lam, case_iterm,
                        case_nelem, rep, Ntot, degen, nslot, N, Kp, w, out, grouped, e_out, row0,
                        rset, (int)blockIdx.x);
}

// The Y rows of every unit of a round in one launch: item k has rows
// [items[k].row0, items[k].row0 + items[k].rows) of the grid and of Y.
template <int S>
__global__ void __launch_bounds__(256)
    k_build_y_digits_items(const YItem* __restrict__ items, int nitems, int N, int Kp, int w,
                           uint32_t* __restrict__ out, int grouped, int32_t* __restrict__ e_out,
                           size_t rset) {
  const long long b = blockIdx.x;
  const int lo = find_item(nitems, b, [&](int k) { return items[k].row0; });
  const YItem& it = items[lo];
  if (b - it.row0 >= it.rows) return;  // not a row of any unit (the whole block)
  build_y_digits_row<S>(it.vecs, it.ld, it.ivec, it.ndeg, it.yptr, it.yroot, it.root_case,
                        it.root_lam, it.case_iterm, it.case_nelem, it.rep, it.Ntot, it.ndeg,
                        it.nslot, N, Kp, w, out, grouped, e_out, (size_t)it.row0, rset,
                        (int)(b - it.row0));
}
constexpr int kFusedYMaxKp = 8192;  // 64 KB of shared memory per row

// ------------------------------------------------------------------ host
typedef CUresult (*EncodeTiledFn)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*,
                                  const cuuint64_t*, const cuuint64_t*, const cuuint32_t*,
                                  const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                  CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiledFn encode_fn() {
  static EncodeTiledFn fn = nullptr;
  if (!fn) {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
            cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = reinterpret_cast<EncodeTiledFn>(p);
  }
  return fn;
}

// 3-D map over digit planes [s][rows][K] of bf16 with a (16, box_rows, box_planes) box.
// K elements of each row starting at base, rows ldk elements apart (a K
// segment of longer rows when ldk > K).
bool make_map(CUtensorMap* map, const void* base, int K, int rows, int s, int box_rows,
              int box_planes, int ldk) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)K, (cuuint64_t)rows, (cuuint64_t)s};
  cuuint64_t strides[2] = {(cuuint64_t)ldk * 2, (cuuint64_t)ldk * rows * 2};
  cuuint32_t box[3] = {(cuuint32_t)kBK, (cuuint32_t)box_rows, (cuuint32_t)box_planes};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_32B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// 3-D map over the grouped layout's four-plane groups [nq][rows][4K]: a box is
// the 64 elements (four planes x 16) of one K slice for box_rows rows, in
// 128-byte rows with the 128-byte swizzle.
bool make_map_groups(CUtensorMap* map, const void* base, int K, int rows, int nq, int box_rows,
                     int ldk) {
  EncodeTiledFn fn = encode_fn();
  if (!fn) return false;
  cuuint64_t dims[3] = {(cuuint64_t)K * 4, (cuuint64_t)rows, (cuuint64_t)nq};
  cuuint64_t strides[2] = {(cuuint64_t)ldk * 8, (cuuint64_t)ldk * rows * 8};
  cuuint32_t box[3] = {64, (cuuint32_t)box_rows, 1};
  cuuint32_t es[3] = {1, 1, 1};
  return fn(map, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 3, const_cast<void*>(base), dims, strides, box,
            es, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B,
            CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// One launch configuration of the split GEMM: the kernel (one pass with all
// diagonals in tensor memory, or two passes with wider tiles) and the L2
// raster group (row tiles whose digit planes share about ga_mb MB of L2).
struct GemmConfig {
  int kind = 1;  // 0: k_split_gemm (one pass); 1, 2: k_split_gemm2 (two passes,
                 // diagonals split at s/2 or s - s/2); these read the plain
                 // layout.  6, 7, 8: k_split_gemm_g on the grouped layout (two
                 // passes split at s/2 or s - s/2, or one pass); 9: its 2-SM
                 // pair form (256-row tiles, two passes split at s/2, s = 9).
                 // 3-5 are unused.
  int ga_mb = 64;
};

// Two-pass geometry: diagonals [0, S/2) then [S/2, S), each pass's accumulators
// within the 512 tensor-memory columns, at most 128 wide.
__host__ __device__ constexpr int d1_of(int s) { return s / 2; }
// the other split point for odd s: the larger half of the diagonals first
__host__ __device__ constexpr int d1b_of(int s) { return s - s / 2; }
__host__ __device__ constexpr int bn2_of(int s) {
  return ((512 / (s - s / 2)) / 16 * 16) > 128 ? 128 : ((512 / (s - s / 2)) / 16 * 16);
}
size_t smemg_bytes(int s, int bn) {
  const size_t need = (size_t)kStages2 * stage_bytes_g(s, bn) + 1024 + 256;
  return need < (size_t)120 * 1024 ? (size_t)120 * 1024 : need;  // one CTA per SM
}
// the 2-SM pair: each CTA stages 128 A rows and bn/2 B rows, in kStagesP slots
size_t smemp_bytes(int s, int bn) {
  return (size_t)kStagesP * stage_bytes_g(s, bn / 2) + 1024 + 256;
}
size_t smem2_bytes(int s, int bn) {
  const size_t need = (size_t)kStages2 * s * (kBM + bn) * kBK * 2 + 1024 + 256;
  return need < (size_t)120 * 1024 ? (size_t)120 * 1024 : need;  // one CTA per SM
}

int tile_n(int s, int kind) { return (kind == 0 || kind == 8) ? bn_for(s) : bn2_of(s); }
// Kernels that read the context's digit layout (grouped needs s >= 4; below
// that the grouped layout is the plain one).
bool kind_valid(int s, int kind, bool grouped) {
  if (grouped && s >= 4)
    return kind == 6 || kind == 8 || (kind == 7 && (s & 1)) || (kind == 9 && s == 9);
  return kind == 0 || kind == 1 || (kind == 2 && (s & 1));
}
GemmConfig default_config(int s, bool grouped) {
  GemmConfig g;
  g.kind = (grouped && s >= 4) ? 6 : 1;
  return g;
}
struct Maps {
  CUtensorMap a, b;    // plain planes, or the grouped layout's four-plane groups
  CUtensorMap at, bt;  // grouped layout: the s % 4 plain planes after the groups
};

SplitShape shape_of(const Ctx* c) {
  int s = c->params.split_slices > 0 ? c->params.split_slices : kDefaultSlices;
  s = std::min(std::max(s, 2), kMaxSlices);
  return SplitShape{s, kDefaultW, tile_n(s, 6)};
}

// Dynamic shared memory above 48 KB must be enabled per kernel, once, before
// the first launch (and before any graph capture).
template <class F>
cudaError_t set_smem(F a, size_t bytes, F b) {
  cudaError_t e = cudaFuncSetAttribute(a, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
  return e != cudaSuccess ? e
                          : cudaFuncSetAttribute(b, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                                 (int)bytes);
}

template <int S>
cudaError_t set_attributes() {
  constexpr int BN1 = bn_for(S), BN2 = bn2_of(S), D1 = d1_of(S);
  static std::once_flag once;
  static cudaError_t status = cudaSuccess;
  std::call_once(once, [] {
    status = cudaFuncSetAttribute(k_split_gemm<S, BN1>,
                                  cudaFuncAttributeMaxDynamicSharedMemorySize,
                                  (int)smem_bytes(S, BN1));
    if (status == cudaSuccess)
      status = cudaFuncSetAttribute(k_split_gemm2<S, BN2, D1>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem2_bytes(S, BN2));
    if (status == cudaSuccess && d1b_of(S) != D1)
      status = cudaFuncSetAttribute(k_split_gemm2<S, BN2, d1b_of(S)>,
                                    cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)smem2_bytes(S, BN2));
    if constexpr (S >= 4) {
      if (status == cudaSuccess)
        status = set_smem(k_split_gemm_g<S, BN2, D1, false>, smemg_bytes(S, BN2), k_split_gemm_g<S, BN2, D1, true>);
      if (status == cudaSuccess && d1b_of(S) != D1)
        status = set_smem(k_split_gemm_g<S, BN2, d1b_of(S), false>, smemg_bytes(S, BN2), k_split_gemm_g<S, BN2, d1b_of(S), true>);
      if (status == cudaSuccess)
        status = set_smem(k_split_gemm_g<S, BN1, S, false>, smemg_bytes(S, BN1), k_split_gemm_g<S, BN1, S, true>);
      if (status == cudaSuccess)
        status = cudaFuncSetAttribute(k_split_gemm_g<S, BN1, S, false, true>,
                                      cudaFuncAttributeMaxDynamicSharedMemorySize,
                                      (int)smemg_bytes(S, BN1));
      if constexpr (S == 9) {
        if (status == cudaSuccess)
          status = cudaFuncSetAttribute(k_split_gemm_gp<S, BN2, D1>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)smemg_bytes(S, BN2));
        if (status == cudaSuccess)
          status = set_smem(k_split_gemm_g<S, BN2, D1, false, false, true>, smemp_bytes(S, BN2),
                            k_split_gemm_g<S, BN2, D1, true, false, true>);
        if (status == cudaSuccess)
          status = cudaFuncSetAttribute(k_build_y_digits<S>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(kFusedYMaxKp * sizeof(double)));
        if (status == cudaSuccess)
          status = cudaFuncSetAttribute(k_build_y_digits_items<S>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)(kFusedYMaxKp * sizeof(double)));
      }
    }
  });
  return status;
}

cudaError_t kernel_attributes(int s) {
  switch (s) {
#define GI_S(SS) \
  case SS: return set_attributes<SS>();
    GI_S(2) GI_S(3) GI_S(4) GI_S(5) GI_S(6) GI_S(7) GI_S(8) GI_S(9) GI_S(10)
#undef GI_S
  }
  return cudaErrorInvalidValue;
}

// kparts > 1 (grouped kernels only): K in parts of kpart_steps 16-wide steps,
// part p writing its own product to C + p * strideP (grid y).
template <int S>
cudaError_t launch_gemm(const GemmConfig& cfg, const Maps& mp, const int32_t* ea,
                        const int32_t* eb, double* C, int ldc, size_t strideC, int M, int Mpad,
                        int Nc, int K, int batch, int w, int accum, int* err,
                        cudaStream_t st, int kparts = 1, int kpart_steps = 0,
                        size_t strideP = 0) {
  const CUtensorMap& tA = mp.a;
  const CUtensorMap& tB = mp.b;
  const bool one = cfg.kind == 0 || cfg.kind == 8;
  constexpr int BN1 = bn_for(S), BN2 = bn2_of(S), D1 = d1_of(S);
  const int BN = one ? BN1 : BN2;
  const size_t sm = cfg.kind == 0 ? smem_bytes(S, BN1)
                    : cfg.kind >= 6 ? smemg_bytes(S, BN) : smem2_bytes(S, BN);
  cudaError_t e = set_attributes<S>();
  if (e != cudaSuccess) return e;
  const int nM = (M + kBM - 1) / kBM, nN = (Nc + BN - 1) / BN, nA = nM * batch;
  // row tiles per L2 group: their digit planes (128 x K x S bf16 each) within ga_mb MB
  const size_t a_tile = (size_t)kBM * K * S * 2;
  const int GA = std::max(1, std::min(nA, (int)(((size_t)cfg.ga_mb << 20) / a_tile)));
  if constexpr (S == 9) {
    if (cfg.kind == 9) {  // 2-SM pairs: clusters of two CTAs, 256-row tiles
      if (kparts > 1) return cudaErrorInvalidValue;
      const int nM2 = (M + 2 * kBM - 1) / (2 * kBM), nA2 = nM2 * batch;
      const int GA2 = std::max(1, std::min(nA2, (int)(((size_t)cfg.ga_mb << 20) / (2 * a_tile))));
      cudaLaunchConfig_t lc = {};
      lc.gridDim = dim3((unsigned)(2 * nA2 * nN));
      lc.blockDim = dim3(kThreadsG);
      lc.dynamicSmemBytes = smemp_bytes(S, BN2);
      lc.stream = st;
      cudaLaunchAttribute at[1];
      at[0].id = cudaLaunchAttributeClusterDimension;
      at[0].val.clusterDim.x = 2;
      at[0].val.clusterDim.y = 1;
      at[0].val.clusterDim.z = 1;
      lc.attrs = at;
      lc.numAttrs = 1;
      auto kern = accum ? k_split_gemm_g<S, BN2, D1, true, false, true>
                        : k_split_gemm_g<S, BN2, D1, false, false, true>;
      return cudaLaunchKernelEx(&lc, kern, mp.a, mp.at, mp.b, mp.bt, ea, eb, C, ldc, strideC, M,
                                Mpad, Nc, K, w, nM2, nA2, nN, GA2, err, 0, (size_t)0);
    }
  }
  if constexpr (S >= 4) {
    if (cfg.kind >= 6 && cfg.kind <= 8) {
      const dim3 grid((unsigned)(nA * nN), (unsigned)std::max(kparts, 1));
      if (kparts > 1) {  // K parts: the one-pass kernel only
        if (cfg.kind != 8 || accum) return cudaErrorInvalidValue;
        k_split_gemm_g<S, BN1, S, false, true><<<grid, kThreadsG, sm, st>>>(
            mp.a, mp.at, mp.b, mp.bt, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA,
            err, kpart_steps, strideP);
        return cudaGetLastError();
      }
      if (cfg.kind == 8)
        (accum ? k_split_gemm_g<S, BN1, S, true> : k_split_gemm_g<S, BN1, S, false>)<<<grid, kThreadsG, sm, st>>>(
            mp.a, mp.at, mp.b, mp.bt, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA,
            err, kpart_steps, strideP);
      else if (cfg.kind == 7 && d1b_of(S) != D1)
        (accum ? k_split_gemm_g<S, BN2, d1b_of(S), true> : k_split_gemm_g<S, BN2, d1b_of(S), false>)<<<grid, kThreadsG, sm, st>>>(
            mp.a, mp.at, mp.b, mp.bt, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA,
            err, kpart_steps, strideP);
      else
        (accum ? k_split_gemm_g<S, BN2, D1, true> : k_split_gemm_g<S, BN2, D1, false>)<<<grid, kThreadsG, sm, st>>>(
            mp.a, mp.at, mp.b, mp.bt, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA,
            err, kpart_steps, strideP);
      return cudaGetLastError();
    }
  }
  if (kparts > 1) return cudaErrorInvalidValue;  // the plain-layout kernels take whole K
  if (one)
    k_split_gemm<S, BN1><<<nA * nN, kThreads, sm, st>>>(
        tA, tB, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA, accum, err);
  else if (cfg.kind == 2 && d1b_of(S) != D1)
    k_split_gemm2<S, BN2, d1b_of(S)><<<nA * nN, kThreads, sm, st>>>(
        tA, tB, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA, accum, err);
  else
    k_split_gemm2<S, BN2, D1><<<nA * nN, kThreads, sm, st>>>(
        tA, tB, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, w, nM, nA, nN, GA, accum, err);
  return cudaGetLastError();
}

cudaError_t launch_gemm_s(int s, const GemmConfig& cfg, const Maps& mp, const int32_t* ea,
                          const int32_t* eb, double* C, int ldc, size_t strideC, int M, int Mpad,
                          int Nc, int K, int batch, int w, int accum, int* err,
                          cudaStream_t st, int kparts = 1, int kpart_steps = 0,
                          size_t strideP = 0) {
  switch (s) {
#define GI_S(SS)                                                                                \
  case SS:                                                                                      \
    return launch_gemm<SS>(cfg, mp, ea, eb, C, ldc, strideC, M, Mpad, Nc, K, batch, w, accum, err, \
                            st, kparts, kpart_steps, strideP);
    GI_S(2) GI_S(3) GI_S(4) GI_S(5) GI_S(6) GI_S(7) GI_S(8) GI_S(9) GI_S(10)
#undef GI_S
  }
  return cudaErrorInvalidValue;
}

cudaError_t slice(const double* X, int ldx, int rows, int K, int rows_pad, int s, int w,
                  bool grouped, uint16_t* out, int32_t* e, cudaStream_t st, int nstack = 1,
                  size_t xstride = 0) {
  if (rows_pad <= 0) return cudaSuccess;
  const int wpb = 8;
  if ((K & 1) || (grouped && (K & 15)) || nstack < 1 || nstack > 65535)
    return cudaErrorInvalidValue;
  if (s == 9) {
    k_slice_rows_b<9><<<dim3(rows_pad, nstack), 256, 0, st>>>(
        X, ldx, xstride, rows, K, rows_pad, w, reinterpret_cast<uint32_t*>(out), grouped ? 1 : 0,
        e);
    return cudaGetLastError();
  }
  const dim3 grid((rows_pad + wpb - 1) / wpb, nstack);
  k_slice_rows<<<grid, wpb * 32, 0, st>>>(X, ldx, xstride, rows, K, rows_pad, s, w,
                                          reinterpret_cast<uint32_t*>(out), grouped ? 1 : 0, e);
  return cudaGetLastError();
}

// Digit layout of a context: grouped (128-byte TMA rows) unless
// GI_SPLIT_LAYOUT=plain asks for the plain plane-by-plane layout.
bool grouped_layout() {
  const char* e = getenv("GI_SPLIT_LAYOUT");
  return !(e && std::strcmp(e, "plain") == 0);
}

}  // namespace

// Per-context state of the split path.
struct SplitState {
  int s = 0, w = 0;
  bool grouped = true;                        // digit layout of every operand
  int N = -1;                                 // dipole the slices belong to
  int panel = 0;                              // rows per panel of a streamed dipole
  DevArray<uint16_t> mu_slices;      // [s][3*Mpad][Kp]
  DevArray<int32_t> mu_exp;                   // [3*Mpad]
  int Mpad = 0;
  DevArray<uint16_t> b_slices;       // workspace: [s][rows][K]
  DevArray<int32_t> b_exp;
  DevArray<uint16_t> v_slices;       // workspace for the final-state vectors
  DevArray<int32_t> v_exp;
  DevArray<int> err;
};

static SplitState* state(Ctx* c) {
  if (!c->split) c->split = new SplitState();
  return c->split;
}

static gi_status check(Ctx* c, cudaError_t e, const char* what) {
  if (e == cudaSuccess) return GI_OK;
  c->err = std::string("split precision: ") + what + ": " + cudaGetErrorString(e);
  return e == cudaErrorMemoryAllocation ? GI_ERR_NOMEM : GI_ERR_CUDA;
}

gi_status split_prepare(Ctx* c) {
  SplitState* S = state(c);
  const SplitShape sh = shape_of(c);
  if (!encode_fn()) {
    c->err = "split precision: cuTensorMapEncodeTiled unavailable";
    return GI_ERR_CUDA;
  }
  gi_status g = check(c, S->err.reserve(1), "error word");
  if (g != GI_OK) return g;
  g = check(c, cudaMemsetAsync(S->err.p, 0, sizeof(int), c->stream), "error word");
  if (g != GI_OK) return g;
  if (c->parent) {
    // a serving worker uses its parent's dipole digits (cut before admission)
    const SplitState* P = c->parent->split;
    if (!P || P->N != c->N || P->s != sh.s || P->w != sh.w) {
      c->err = "split precision: the dipole digits of the serving context are not prepared";
      return GI_ERR_STATE;
    }
    S->s = P->s;
    S->w = P->w;
    S->N = P->N;
    S->Mpad = P->Mpad;
    S->grouped = P->grouped;
    return GI_OK;
  }
  const bool grouped = grouped_layout();
  const int P = dipole_panel_rows(c);  // 0: the dipole is resident
  if (S->N == c->N && S->s == sh.s && S->w == sh.w && S->grouped == grouped && S->panel == P)
    return GI_OK;
  S->grouped = grouped;
  S->s = sh.s;
  S->w = sh.w;
  S->panel = P;
  // digit planes of the dipole (of one panel when streamed): rows = 3
  // components x Mpad, K = Kp
  S->Mpad = round_up(P ? P : c->N, kBM);
  const size_t rows = (size_t)3 * S->Mpad;
  if (S->mu_slices.n != (size_t)sh.s * rows * c->Kp) {  // same shape: recut in place
    g = check(c, S->mu_slices.alloc((size_t)sh.s * rows * c->Kp), "dipole slices");
    if (g != GI_OK) return g;
  }
  if (S->mu_exp.n != rows) {
    g = check(c, S->mu_exp.alloc(rows), "dipole exponents");
    if (g != GI_OK) return g;
  }
  if (P) {  // a streamed panel is cut before its GEMM
    S->N = c->N;
    return GI_OK;
  }
  // all three components in one launch: [3][N][Kp] -> the [3 Mpad]-row set
  g = check(c,
            slice(c->d_mu.p, c->Kp, c->N, c->Kp, S->Mpad, sh.s, sh.w, grouped, S->mu_slices.p,
                  S->mu_exp.p, c->stream, 3, (size_t)c->N * c->Kp),
            "slice dipole");
  if (g != GI_OK) return g;
  g = check(c, cudaStreamSynchronize(c->stream), "slice dipole sync");
  if (g != GI_OK) return g;
  S->N = c->N;
  return GI_OK;
}

// ------------------------------------------------------------------ autotuner
// The launch configuration is chosen per GEMM shape class (digits, row tiles,
// power-of-two column bucket, K).  With tuning on, the first GEMM of a class
// times every candidate on its real operands with CUDA events and keeps the
// fastest; the table lives for the process and, given a path, in a text file
// ("s nA nbucket K layout kind ga_mb ms" per line).
struct TuneKey {
  int s, nA, nbucket, K, layout;
  bool operator<(const TuneKey& o) const {
    return std::tie(s, nA, nbucket, K, layout) < std::tie(o.s, o.nA, o.nbucket, o.K, o.layout);
  }
};
struct TuneEntry {
  GemmConfig cfg;
  float ms;
};
struct Tuner {
  std::mutex mu;
  std::map<TuneKey, TuneEntry> table;
  std::string loaded;
  uint64_t version = 0;  // bumped on every change (captured graphs depend on it)
};
static Tuner& tuner() {
  static Tuner t;
  return t;
}
static const GemmConfig kCandidates[] = {{1, 64}, {1, 32}, {1, 128}, {1, 16}, {2, 64},
                                         {2, 32}, {0, 64}, {0, 32}, {6, 64}, {6, 32},
                                         {6, 128}, {7, 64}, {7, 32}, {8, 64}, {8, 32},
                                         {9, 64}, {9, 32}, {9, 128}};

static void tune_load(Tuner& t, const std::string& path) {
  t.loaded = path;
  FILE* f = fopen(path.c_str(), "r");
  if (!f) return;
  TuneKey k;
  TuneEntry e;
  while (fscanf(f, "%d %d %d %d %d %d %d %f", &k.s, &k.nA, &k.nbucket, &k.K, &k.layout,
                &e.cfg.kind, &e.cfg.ga_mb, &e.ms) == 8)
    if (kind_valid(k.s, e.cfg.kind, k.layout != 0) && e.cfg.ga_mb > 0) t.table[k] = e;
  fclose(f);
  t.version++;
}

static void tune_save(const Tuner& t, const std::string& path) {
  const std::string tmp = path + ".tmp";
  FILE* f = fopen(tmp.c_str(), "w");
  if (!f) return;
  for (const auto& kv : t.table)
    fprintf(f, "%d %d %d %d %d %d %d %.4f\n", kv.first.s, kv.first.nA, kv.first.nbucket,
            kv.first.K, kv.first.layout, kv.second.cfg.kind, kv.second.cfg.ga_mb, kv.second.ms);
  fclose(f);
  rename(tmp.c_str(), path.c_str());
}

static int col_bucket(int n) {
  int b = 0;
  while (b < 30 && (2 << b) <= n) b++;
  return b;
}

static gi_status gemm(Ctx* c, const uint16_t* Aslices, int Arows_total, const int32_t* ea,
                      int Mpad, const uint16_t* Bslices, int Brows, const int32_t* eb,
                      double* C, int ldc, size_t strideC, int M, int Nc, int K, int batch) {
  SplitState* S = state(c);
  const bool grouped = S->grouped && S->s >= 4;
  // K runs in segments of at most kKSeg, each a launch whose FP64 results
  // the next adds to: within a segment every diagonal sum that carries weight
  // stays an exact fp32 integer (the bound in the header); the segments are
  // summed in FP64.
  const int nseg = (K + kKSeg - 1) / kKSeg;
  c->stats.kernel_launches += nseg - 1;
  auto run = [&](const GemmConfig& g) -> cudaError_t {
    const int bn = tile_n(S->s, g.kind);
    const int bbox = g.kind == 9 ? bn / 2 : bn;  // B rows one CTA loads
    for (int k0 = 0; k0 < K; k0 += kKSeg) {
      const int Kc = std::min(kKSeg, K - k0);
      Maps mp;
      if (grouped) {
        // a K segment of the grouped rows starts 4 * k0 elements in (k0 % 16 == 0)
        const int nq = S->s / 4, nt = S->s % 4;
        const uint16_t* At = Aslices + (size_t)4 * nq * Arows_total * K + k0;
        const uint16_t* Bt = Bslices + (size_t)4 * nq * Brows * K + k0;
        if (!make_map_groups(&mp.a, Aslices + (size_t)4 * k0, Kc, Arows_total, nq, kBM, K) ||
            !make_map_groups(&mp.b, Bslices + (size_t)4 * k0, Kc, Brows, nq, bbox, K))
          return cudaErrorInvalidValue;
        if (nt) {
          if (!make_map(&mp.at, At, Kc, Arows_total, nt, kBM, 1, K) ||
              !make_map(&mp.bt, Bt, Kc, Brows, nt, bbox, 1, K))
            return cudaErrorInvalidValue;
        } else {
          mp.at = mp.a;  // no plain planes: never read
          mp.bt = mp.b;
        }
      } else {
        const int planes = g.kind == 0 ? S->s : 1;  // the two-pass kernels load plane by plane
        if (!make_map(&mp.a, Aslices + k0, Kc, Arows_total, S->s, kBM, planes, K) ||
            !make_map(&mp.b, Bslices + k0, Kc, Brows, S->s, bn, planes, K))
          return cudaErrorInvalidValue;
      }
      const cudaError_t e = launch_gemm_s(S->s, g, mp, ea, eb, C, ldc, strideC, M, Mpad, Nc, Kc,
                                          batch, S->w, k0 > 0, S->err.p, c->stream);
      if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
  };
  const TuneKey key{S->s, ((M + kBM - 1) / kBM) * batch, col_bucket(Nc), K, (int)grouped};
  GemmConfig cfg = default_config(S->s, grouped);
  bool known = false;
  // GI_SPLIT_FORCE="kind:ga_mb" pins one configuration (parity tests of every kernel)
  if (const char* f = getenv("GI_SPLIT_FORCE")) {
    GemmConfig g;
    if (sscanf(f, "%d:%d", &g.kind, &g.ga_mb) == 2 && kind_valid(S->s, g.kind, grouped) &&
        g.ga_mb > 0)
      return check(c, run(g), "split GEMM launch");
  }
  Tuner& t = tuner();
  {
    std::lock_guard<std::mutex> lk(t.mu);
    if (!c->tune_path.empty() && t.loaded != c->tune_path) tune_load(t, c->tune_path);
    auto it = t.table.find(key);
    if (it != t.table.end()) {
      cfg = it->second.cfg;
      known = true;
    }
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (!known && c->tune_mode > 0 && cudaStreamIsCapturing(c->stream, &cs) == cudaSuccess &&
      cs == cudaStreamCaptureStatusNone) {
    cudaEvent_t a = nullptr, b = nullptr;
    gi_status g = check(c, cudaEventCreate(&a), "tuning event");
    if (g == GI_OK) g = check(c, cudaEventCreate(&b), "tuning event");
    if (g == GI_OK) g = check(c, run(cfg), "tuning warm-up");  // the first launch of a shape
    float best = 1e30f;
    GemmConfig best_cfg = cfg;
    for (const GemmConfig& cand : kCandidates) {
      if (g != GI_OK) break;
      if (!kind_valid(S->s, cand.kind, grouped)) continue;
      g = check(c, cudaEventRecord(a, c->stream), "tuning event");
      if (g == GI_OK) g = check(c, run(cand), "tuning launch");
      if (g == GI_OK) g = check(c, cudaEventRecord(b, c->stream), "tuning event");
      if (g == GI_OK) g = check(c, cudaEventSynchronize(b), "tuning sync");
      float ms = 0.f;
      if (g == GI_OK) g = check(c, cudaEventElapsedTime(&ms, a, b), "tuning time");
      if (g == GI_OK && ms < best) {
        best = ms;
        best_cfg = cand;
      }
    }
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (g != GI_OK) return g;
    std::lock_guard<std::mutex> lk(t.mu);
    t.table[key] = TuneEntry{best_cfg, best};
    t.version++;
    if (!c->tune_path.empty()) tune_save(t, c->tune_path);
    cfg = best_cfg;
  }
  return check(c, run(cfg), "split GEMM launch");
}

gi_status split_gemm_dipole(Ctx* c, const double* Y, int ldy, double* Z, int ldz, size_t zstride,
                            int ncol, bool y_digits_ready) {
  SplitState* S = state(c);
  const int K = c->Kp;
  gi_status g = check(c, S->b_slices.reserve((size_t)S->s * ncol * K), "Y slices");
  if (g != GI_OK) return g;
  g = check(c, S->b_exp.reserve(ncol), "Y exponents");
  if (g != GI_OK) return g;
  if (!y_digits_ready) {
    g = check(c, timed(c, GI_PHASE_SLICE, [&] {
                return slice(Y, ldy, ncol, K, ncol, S->s, S->w, S->grouped, S->b_slices.p,
                             S->b_exp.p, c->stream);
              }),
              "slice Y");
    if (g != GI_OK) return g;
  }
  // algorithmic count: the true contraction length N, not the padded K
  c->stats.flops_tensor += (double)S->s * (S->s + 1) / 2 * 2.0 * c->N * (double)ncol * c->N * 3;
  if (S->panel) {
    // streamed dipole: cut each panel's digits, then its rows [f0, f0 + rows) of Z
    return for_each_dipole_panel(c, c->stream, [&](const double* mu, size_t ms, int rows,
                                                   int f0) -> gi_status {
      gi_status q = check(c, timed(c, GI_PHASE_SLICE, [&] {
                            return slice(mu, K, rows, K, S->Mpad, S->s, S->w, S->grouped,
                                         S->mu_slices.p, S->mu_exp.p, c->stream, 3, ms);
                          }),
                          "slice dipole panel");
      if (q != GI_OK) return q;
      timed(c, GI_PHASE_HALFLS_GEMM, [&] {
        q = gemm(c, S->mu_slices.p, 3 * S->Mpad, S->mu_exp.p, S->Mpad, S->b_slices.p, ncol,
                 S->b_exp.p, Z + f0, ldz, zstride, rows, ncol, K, 3);
        return cudaSuccess;
      });
      return q;
    });
  }
  gi_status r = GI_OK;
  cudaError_t e = timed(c, GI_PHASE_HALFLS_GEMM, [&] {
    const SplitState* D = c->parent ? c->parent->split : S;  // owner of the dipole digits
    r = gemm(c, D->mu_slices.p, 3 * S->Mpad, D->mu_exp.p, S->Mpad, S->b_slices.p, ncol,
             S->b_exp.p, Z, ldz, zstride, c->N, ncol, K, 3);
    return cudaSuccess;
  });
  (void)e;
  return r;
}

// The final-state vectors are fixed inputs: their digits are cut once and
// kept with the block until it is replaced.  Serving workers share blocks, so
// the cut happens under the model lock and the others wait on its event.
static gi_status block_digits(Ctx* c, Block& fb, int K, bool wait) {
  SplitState* S = state(c);
  const int nvec = fb.nvec;
  const int vpad = round_up(nvec, kBM);
  gi_status g;
  std::lock_guard<std::mutex> lk(c->mmu());
  if (fb.digits_s != S->s || fb.digits_w != S->w || fb.digits_layout != (int)S->grouped) {
    const size_t nd = (size_t)S->s * vpad * K;  // same shape: recut in place
    if (fb.d_digits.n != nd) {
      g = check(c, fb.d_digits.alloc(nd), "V digits");
      if (g != GI_OK) return g;
    }
    if (fb.d_digit_exp.n != (size_t)vpad) {
      g = check(c, fb.d_digit_exp.alloc(vpad), "V exponents");
      if (g != GI_OK) return g;
    }
    g = check(c, timed(c, GI_PHASE_SLICE, [&] {
                return slice(fb.d_vecs.p, fb.ld, nvec, K, vpad, S->s, S->w, S->grouped, fb.d_digits.p,
                             fb.d_digit_exp.p, c->stream);
              }),
              "slice V");
    if (g != GI_OK) return g;
    if (!fb.digits_ev) {
      g = check(c, cudaEventCreateWithFlags(&fb.digits_ev, cudaEventDisableTiming), "event");
      if (g != GI_OK) return g;
    }
    g = check(c, cudaEventRecord(fb.digits_ev, c->stream), "event");
    if (g != GI_OK) return g;
    fb.digits_s = S->s;
    fb.digits_w = S->w;
    fb.digits_layout = (int)S->grouped;
  }
  if (wait && fb.digits_ev) {
    // inside a graph capture the cut precedes the capture on this stream
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    g = check(c, cudaStreamIsCapturing(c->stream, &cs), "capture status");
    if (g != GI_OK) return g;
    if (cs == cudaStreamCaptureStatusNone) {
      g = check(c, cudaStreamWaitEvent(c->stream, fb.digits_ev, 0), "event wait");
      if (g != GI_OK) return g;
    }
  }
  return GI_OK;
}

gi_status split_reserve(Ctx* c, size_t max_elems, size_t max_cols,
                        const std::vector<Block*>& finals) {
  SplitState* S = state(c);
  gi_status g = check(c, S->b_slices.reserve((size_t)S->s * max_elems), "B slices");
  if (g != GI_OK) return g;
  g = check(c, S->b_exp.reserve(std::max<size_t>(max_cols, 1)), "B exponents");
  if (g != GI_OK) return g;
  for (Block* b : finals) {
    g = block_digits(c, *b, b->ld, false);
    if (g != GI_OK) return g;
  }
  return check(c, kernel_attributes(S->s), "kernel attributes");
}

gi_status split_gemm_final(Ctx* c, Block& fb, const double* H, int ldh, int ncol, double* T,
                           int ldt) {
  SplitState* S = state(c);
  const int K = ldh;
  const int nvec = fb.nvec;
  const int vpad = round_up(nvec, kBM);
  gi_status g;
  g = block_digits(c, fb, K, /*wait=*/true);
  if (g != GI_OK) return g;
  g = check(c, S->b_slices.reserve((size_t)S->s * ncol * K), "H slices");
  if (g != GI_OK) return g;
  g = check(c, S->b_exp.reserve(ncol), "H exponents");
  if (g != GI_OK) return g;
  g = check(c, timed(c, GI_PHASE_SLICE, [&] {
              return slice(H, ldh, ncol, K, ncol, S->s, S->w, S->grouped, S->b_slices.p, S->b_exp.p,
                           c->stream);
            }),
            "slice H");
  if (g != GI_OK) return g;
  c->stats.flops_tensor += (double)S->s * (S->s + 1) / 2 * 2.0 * nvec * (double)ncol * fb.nsize;
  gi_status r = GI_OK;
  timed(c, GI_PHASE_FINAL_GEMM, [&] {
    r = gemm(c, fb.d_digits.p, vpad, fb.d_digit_exp.p, vpad, S->b_slices.p, ncol, S->b_exp.p, T,
             ldt, 0, nvec, ncol, K, 1);
    return cudaSuccess;
  });
  return r;
}

// The persistent grouped final GEMM: the default two-pass grouped geometry at
// s = 9 (other digit counts, the plain layout and a pinned GI_SPLIT_FORCE
// configuration take one launch per final block); GI_SPLIT_PERSIST=0 turns it
// off.
bool split_grouped_final(const Ctx* c) {
  if (!c->split || !c->split->grouped || c->split->s != 9 || getenv("GI_SPLIT_FORCE"))
    return false;
  const char* e = getenv("GI_SPLIT_PERSIST");
  return !(e && std::strcmp(e, "0") == 0);
}
int split_grouped_max_jobs() { return kGpMaxProb; }
int split_grouped_items(int nvec, int ncol) {
  return (round_up(nvec, kBM) / kBM) * ((ncol + bn2_of(9) - 1) / bn2_of(9));
}

bool split_fused_epilogue(const Ctx* c) {
  if (!split_grouped_final(c)) return false;
  const char* e = getenv("GI_SPLIT_FUSED_EPI");
  return !(e && std::strcmp(e, "0") == 0);
}

gi_status split_gemm_final_grouped(Ctx* c, const std::vector<FinalJob>& jobs,
                                   const FusedLines* lines) {
  SplitState* S = state(c);
  constexpr int SS = 9, BN = bn2_of(SS), D1 = d1_of(SS);
  if (S->s != SS || !S->grouped || jobs.empty() || (int)jobs.size() > kGpMaxProb) {
    c->err = "split precision: grouped final GEMM outside its configuration";
    return GI_ERR_STATE;
  }
  gi_status g;
  size_t elems = 0, cols = 0;
  for (const FinalJob& j : jobs) {
    elems += (size_t)j.ncol * j.ldh;
    cols += j.ncol;
  }
  g = check(c, S->b_slices.reserve((size_t)SS * elems), "H slices");
  if (g != GI_OK) return g;
  g = check(c, S->b_exp.reserve(std::max<size_t>(cols, 1)), "H exponents");
  if (g != GI_OK) return g;
  // problems in decreasing K, so that the longest items are dealt out first
  std::vector<int> order(jobs.size());
  for (size_t i = 0; i < jobs.size(); ++i) order[i] = (int)i;
  std::stable_sort(order.begin(), order.end(),
                   [&](int a, int b) { return jobs[a].ldh > jobs[b].ldh; });
  GpParams* P = new GpParams();  // ~28 KB: not on the host stack
  P->nprob = (int)jobs.size();
  P->nitems = 0;
  P->fused = lines ? 1 : 0;
  if (lines) {
    P->out = lines->out;
    P->counter = lines->counter;
    P->cap = lines->cap;
    P->rec = lines->rec;
    P->rec_cap = lines->rec_cap;
  }
  size_t eoff = 0, boff = 0;
  double flops = 0.0;
  // the H rows of every problem are cut in one launch (GI_BATCH_SMALL=0: one
  // launch per problem)
  const char* bs_env = getenv("GI_BATCH_SMALL");
  const bool batch = !(bs_env && bs_env[0] == '0');
  SliceOps* ops = new SliceOps();
  ops->n = 0;
  ops->row0[0] = 0;
  for (int q = 0; q < (int)jobs.size() && g == GI_OK; ++q) {
    const FinalJob& j = jobs[order[q]];
    Block& fb = *j.fb;
    const int K = j.ldh, vpad = round_up(fb.nvec, kBM);
    g = block_digits(c, fb, K, /*wait=*/true);
    if (g != GI_OK) break;
    uint16_t* bs = S->b_slices.p + boff;
    int32_t* be = S->b_exp.p + eoff;
    if (batch) {
      if (j.ncol > 0) {
        const int o = ops->n++;
        ops->K[o] = K;
        ops->ldx[o] = j.ldh;
        ops->X[o] = j.H;
        ops->out[o] = reinterpret_cast<uint32_t*>(bs);
        ops->e[o] = be;
        ops->row0[o + 1] = ops->row0[o] + j.ncol;
      }
    } else {
      g = check(c, timed(c, GI_PHASE_SLICE, [&] {
                  return slice(j.H, j.ldh, j.ncol, K, j.ncol, SS, S->w, true, bs, be, c->stream);
                }),
                "slice H");
      if (g != GI_OK) break;
    }
    GpProb& pr = P->p[q];
    const int nq = SS / 4, nt = SS % 4;
    if (!make_map_groups(&pr.aq, fb.d_digits.p, K, vpad, nq, kBM, K) ||
        !make_map(&pr.at, fb.d_digits.p + (size_t)4 * nq * vpad * K, K, vpad, nt, kBM, 1, K) ||
        !make_map_groups(&pr.bq, bs, K, j.ncol, nq, BN, K) ||
        !make_map(&pr.bt, bs + (size_t)4 * nq * j.ncol * K, K, j.ncol, nt, BN, 1, K)) {
      g = check(c, cudaErrorInvalidValue, "grouped final GEMM tensor maps");
      break;
    }
    pr.ea = fb.d_digit_exp.p;
    pr.eb = be;
    pr.C = j.T;
    pr.ldc = j.ldt;
    pr.M = fb.nvec;
    pr.Mpad = vpad;
    pr.Nc = j.ncol;
    pr.K = K;
    pr.nM = vpad / kBM;
    pr.nN = (j.ncol + BN - 1) / BN;
    pr.first = P->nitems;
    pr.parts = j.parts;
    pr.nparts = j.nparts;
    pr.EF = j.EF;
    pr.upper = j.upper;
    pr.lvF = j.lvF;
    if (lines && (!j.parts || j.nparts <= 0)) {
      g = check(c, cudaErrorInvalidValue, "fused epilogue without parts");
      break;
    }
    P->nitems += pr.nM * pr.nN;
    boff += (size_t)SS * j.ncol * K;
    eoff += j.ncol;
    flops += (double)SS * (SS + 1) / 2 * 2.0 * fb.nvec * (double)j.ncol * fb.nsize;
  }
  if (g == GI_OK && ops->n > 0) {
    for (int o = 0; o < ops->n; ++o)  // the grouped layout cuts K in 16-element slices
      if (ops->K[o] & 15) g = check(c, cudaErrorInvalidValue, "slice H");
    if (g == GI_OK)
      g = check(c, timed(c, GI_PHASE_SLICE, [&] {
                  k_slice_rows_ops<SS><<<ops->row0[ops->n], 256, 0, c->stream>>>(*ops, S->w, 1);
                  return cudaGetLastError();
                }),
                "slice H");
  }
  delete ops;
  if (g == GI_OK && P->nitems > 0) {
    c->stats.flops_tensor += flops;
    g = check(c, kernel_attributes(SS), "kernel attributes");
    if (g == GI_OK) {
      const int grid = std::min(P->nitems, std::max(c->nsm, 1));
      const size_t sm = smemg_bytes(SS, BN);
      g = check(c, timed(c, GI_PHASE_FINAL_GEMM, [&] {
                  k_split_gemm_gp<SS, BN, D1><<<grid, kThreadsG, sm, c->stream>>>(*P, S->w,
                                                                                 S->err.p);
                  return cudaGetLastError();
                }),
                "grouped final GEMM launch");
    }
  }
  delete P;
  return g;
}

// The half line strength of a few vectors: Z = mu^T Y for ncol columns, far
// fewer than one 96-wide tile.  The dipole digits are the data that moves
// (3 x Mpad x Kp x s bf16), so the GEMM is as fast as one pass over them:
// the row tiles alone are too few CTAs to draw full HBM bandwidth, so K is
// split into parts (the grid's y dimension of one launch of the one-pass
// kernel: 48-wide tiles, every diagonal in tensor memory, the dipole digits
// read once), each writing its own partial product Zp[part][col][3 * Mpad];
// the caller sums the parts.  Streamed dipoles and digit shapes other than the default grouped
// s = 9 go through the regular GEMM as one part.
gi_status split_gemm_dipole_narrow(Ctx* c, const double* Y, int ldy, int ncol, double* Zp,
                                   size_t part_stride, int max_parts, int* nparts, int* ldz) {
  SplitState* S = state(c);
  const SplitState* D = c->parent ? c->parent->split : S;
  const int K = c->Kp;
  const int rows = 3 * S->Mpad;
  *ldz = rows;
  if (S->panel) {
    c->err = "split precision: the narrow dipole GEMM needs a resident dipole";
    return GI_ERR_STATE;
  }
  gi_status g = check(c, S->b_slices.reserve((size_t)S->s * ncol * K), "Y slices");
  if (g != GI_OK) return g;
  g = check(c, S->b_exp.reserve(ncol), "Y exponents");
  if (g != GI_OK) return g;
  g = check(c, timed(c, GI_PHASE_SLICE, [&] {
              return slice(Y, ldy, ncol, K, ncol, S->s, S->w, S->grouped, S->b_slices.p,
                           S->b_exp.p, c->stream);
            }),
            "slice Y");
  if (g != GI_OK) return g;
  c->stats.flops_tensor += (double)S->s * (S->s + 1) / 2 * 2.0 * c->N * (double)ncol * c->N * 3;
  constexpr int SS = 9, BN = bn_for(SS);  // the one-pass tile width
  const int nM = rows / kBM, nN = (ncol + BN - 1) / BN;
  // parts: enough to give every SM a tile; each a multiple of 64 in K and at
  // most one exact segment long (a launch does not segment K)
  const int kq = K / 64, pmax = std::max(1, max_parts);
  int parts = std::max(1, std::min({std::max(c->nsm, 1) / (nM * nN), pmax, kq}));
  while (parts < pmax && (kq + parts - 1) / parts * 64 > kKSeg) parts++;
  const int per = (kq + parts - 1) / parts * 64;
  parts = (K + per - 1) / per;  // no empty part
  if (S->s != SS || !S->grouped || getenv("GI_SPLIT_FORCE") || per > kKSeg) {
    *nparts = 1;
    gi_status r = GI_OK;
    timed(c, GI_PHASE_HALFLS_GEMM, [&] {
      r = gemm(c, D->mu_slices.p, rows, D->mu_exp.p, rows, S->b_slices.p, ncol, S->b_exp.p, Zp,
               rows, 0, rows, ncol, K, 1);
      return cudaSuccess;
    });
    return r;
  }
  *nparts = parts;
  // one launch of the one-pass grouped kernel (48-wide tiles, all nine
  // diagonals in tensor memory, so the dipole digits stream through once),
  // the K parts on the grid's y dimension
  const int nq = SS / 4, nt = SS % 4;
  GemmConfig cfg;
  cfg.kind = 8;
  cfg.ga_mb = 64;
  Maps mp;
  if (!make_map_groups(&mp.a, D->mu_slices.p, K, rows, nq, kBM, K) ||
      !make_map(&mp.at, D->mu_slices.p + (size_t)4 * nq * rows * K, K, rows, nt, kBM, 1, K) ||
      !make_map_groups(&mp.b, S->b_slices.p, K, ncol, nq, BN, K) ||
      !make_map(&mp.bt, S->b_slices.p + (size_t)4 * nq * ncol * K, K, ncol, nt, BN, 1, K))
    return check(c, cudaErrorInvalidValue, "narrow dipole GEMM tensor maps");
  return check(c, timed(c, GI_PHASE_HALFLS_GEMM, [&] {
                 return launch_gemm_s(SS, cfg, mp, D->mu_exp.p, S->b_exp.p, Zp, rows, 0, rows,
                                      rows, ncol, K, 1, S->w, 0, S->err.p, c->stream, parts,
                                      per / kBK, part_stride);
               }),
               "narrow dipole GEMM launch");
}

bool split_fused_y(const Ctx* c) { return split_grouped_final(c) && c->Kp <= kFusedYMaxKp; }

gi_status split_build_y_digits_items(Ctx* c, const YItem* items, int n, long long rows,
                                     size_t rows_total) {
  SplitState* S = state(c);
  if (n <= 0 || rows <= 0) return GI_OK;
  if (S->s != 9 || S->b_slices.n < (size_t)9 * rows_total * c->Kp || S->b_exp.n < rows_total ||
      rows > 0x7FFFFFFFll) {
    c->err = "split precision: Y digit workspace not prepared";
    return GI_ERR_STATE;
  }
  return check(c, timed(c, GI_PHASE_CORRELATE, [&] {
                 k_build_y_digits_items<9><<<(unsigned)rows, 256, (size_t)c->Kp * sizeof(double),
                                             c->stream>>>(
                     items, n, c->N, c->Kp, S->w, reinterpret_cast<uint32_t*>(S->b_slices.p),
                     S->grouped ? 1 : 0, S->b_exp.p, rows_total);
                 return cudaGetLastError();
               }),
               "Y digits");
}

gi_status split_build_y_digits(Ctx* c, const double* vecs, int ld, const int32_t* ivec, int nI,
                               int ndeg, const Basis& b, int gamma, size_t row0,
                               size_t rows_total) {
  SplitState* S = state(c);
  const int rows = nI * ndeg * b.nslot;
  if (rows == 0) return GI_OK;
  if (S->s != 9 || S->b_slices.n < (size_t)9 * rows_total * c->Kp || S->b_exp.n < rows_total) {
    c->err = "split precision: Y digit workspace not prepared";
    return GI_ERR_STATE;
  }
  return check(c, timed(c, GI_PHASE_CORRELATE, [&] {
                 k_build_y_digits<9><<<rows, 256, (size_t)c->Kp * sizeof(double), c->stream>>>(
                     vecs, ld, ivec, ndeg, b.d_yptr.p, b.d_yroot.p, b.d_root_case.p,
                     b.d_root_lam.p, b.d_case_iterm[gamma].p, b.d_case_nelem[gamma].p,
                     b.d_rep[gamma].p, b.Ntotal[gamma], ndeg, b.nslot, c->N, c->Kp, S->w,
                     reinterpret_cast<uint32_t*>(S->b_slices.p), S->grouped ? 1 : 0, S->b_exp.p,
                     row0, rows_total);
                 return cudaGetLastError();
               }),
               "Y digits");
}

int split_digits(const Ctx* c) { return shape_of(c).s; }

uint64_t split_identity(Ctx* c) {
  const SplitState* S = state(c);
  const SplitState* D = c->parent ? c->parent->split : S;
  uint64_t h = 1469598103934665603ull;
  for (uint64_t v : {(uint64_t)(uintptr_t)S->b_slices.p, (uint64_t)(uintptr_t)S->b_exp.p,
                     (uint64_t)(uintptr_t)S->err.p, (uint64_t)(uintptr_t)D->mu_slices.p,
                     (uint64_t)(uintptr_t)D->mu_exp.p, (uint64_t)S->s, (uint64_t)S->w,
                     (uint64_t)S->Mpad, tuner().version})
    h = (h ^ v) * 1099511628211ull;
  return h;
}

const int* split_error_word(const Ctx* c) {
  return c->split ? c->split->err.p : nullptr;
}

gi_status split_check(Ctx* c) {
  if (!c->split || !c->split->err.p) return GI_OK;
  int e = 0;
  if (cudaMemcpy(&e, c->split->err.p, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess)
    return GI_ERR_CUDA;
  if (e) {
    char buf[128];
    snprintf(buf, sizeof(buf), "split GEMM: a pipeline wait timed out (code %d)", e);
    c->err = buf;
    return GI_ERR_DEVICE;
  }
  return GI_OK;
}

void split_invalidate(Ctx* c) {
  if (c->split) c->split->N = -1;
}

void split_release(Ctx* c) {
  delete c->split;
  c->split = nullptr;
}

}  // namespace gi

extern "C" gi_status gi_probe_split_gemm(int device, int slices, int M, int N, int K,
                                          const double* A, const double* B, double* C) {
  using namespace gi;
  if (M <= 0 || N <= 0 || K <= 0 || !A || !B || !C) return GI_ERR_ARG;
  if (cudaSetDevice(device) != cudaSuccess) return GI_ERR_CUDA;
  if (!encode_fn()) return GI_ERR_CUDA;
  Ctx c;
  c.device = device;
  c.params.split_slices = slices;
  if (cudaStreamCreateWithFlags(&c.stream, cudaStreamNonBlocking) != cudaSuccess)
    return GI_ERR_CUDA;
  SplitState* S = state(&c);
  const SplitShape sh = shape_of(&c);
  S->s = sh.s;
  S->w = sh.w;
  S->grouped = grouped_layout();
  const int Kp = round_up(K, 64), Mpad = round_up(M, kBM);
  DevArray<double> dA, dB, dC;
  DevArray<uint16_t> sa, sb;
  DevArray<int32_t> xa, xb;
  gi_status g = GI_OK;
  auto ck = [&](cudaError_t e) {
    if (g == GI_OK && e != cudaSuccess)
      g = e == cudaErrorMemoryAllocation ? GI_ERR_NOMEM : GI_ERR_CUDA;
  };
  ck(dA.alloc((size_t)M * Kp));
  ck(dB.alloc((size_t)N * Kp));
  ck(dC.alloc((size_t)N * M));
  ck(sa.alloc((size_t)S->s * Mpad * Kp));
  ck(sb.alloc((size_t)S->s * N * Kp));
  ck(xa.alloc(Mpad));
  ck(xb.alloc(N));
  ck(S->err.reserve(1));
  if (g == GI_OK) {
    ck(cudaMemset(dA.p, 0, sizeof(double) * dA.n));
    ck(cudaMemset(dB.p, 0, sizeof(double) * dB.n));
    ck(cudaMemset(S->err.p, 0, sizeof(int)));
    ck(cudaMemcpy2D(dA.p, sizeof(double) * Kp, A, sizeof(double) * K, sizeof(double) * K, M,
                    cudaMemcpyHostToDevice));
    ck(cudaMemcpy2D(dB.p, sizeof(double) * Kp, B, sizeof(double) * K, sizeof(double) * K, N,
                    cudaMemcpyHostToDevice));
    ck(cudaDeviceSynchronize());
  }
  if (g == GI_OK) {
    ck(slice(dA.p, Kp, M, Kp, Mpad, S->s, S->w, S->grouped, sa.p, xa.p, c.stream));
    ck(slice(dB.p, Kp, N, Kp, N, S->s, S->w, S->grouped, sb.p, xb.p, c.stream));
  }
  if (g == GI_OK) g = gemm(&c, sa.p, Mpad, xa.p, Mpad, sb.p, N, xb.p, dC.p, M, 0, M, N, Kp, 1);
  if (g == GI_OK) ck(cudaStreamSynchronize(c.stream));
  if (g == GI_OK) g = split_check(&c);
  if (g == GI_OK) ck(cudaMemcpy(C, dC.p, sizeof(double) * N * M, cudaMemcpyDeviceToHost));
  cudaStreamSynchronize(c.stream);
  split_release(&c);
  cudaStreamDestroy(c.stream);
  return g;
}
