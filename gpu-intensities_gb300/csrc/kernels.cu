// Gather/scatter, stencil, epilogue and FP64 DMMA GEMM kernels of the
// line-intensity engine (sm_103a).
//
// Factorisation of the reference's half line strength
// (dipole_kernals.cu:162-227).  With keyI = 2kI+tauI, the reference sums
//   h[rF] = sgnF * sum_rI [|kI-kF|<=1] R(keyI,keyF) * mu_c(icontrI, icontrF) * vI[rI]
// where R (sign, L, 3j, 1/sqrt2) and the component c depend only on the two
// keys.  Grouping the initial roots by key gives
//   Y[slotI][v] = sum_{rI: key=slotI, icontrI=v} vI[rI]            (k_build_y)
//   Z_c[slotI][f] = sum_v mu_c(v, f) Y[slotI][v]                    (a GEMM)
//   h[rF] = sum_{terms of keyF} coef * Z_c[slotI][icontrF(rF)]      (k_build_h)
// and the reference's per-final-vector correlate + Ddot (cuda_host.cu:1301-1317)
// becomes a GEMM against H projected back onto the symmetrised basis:
//   H[s] = sum_lambda repres_F[s, idegF, lambda] * h[root(case(s), lambda)].
#include <cuda_runtime.h>

#include <algorithm>

#include "engine.h"
#include "epilogue.cuh"
#include "items.cuh"

namespace gi {

// ------------------------------------------------------------------ Y build
// One thread per (slot, v) element of one column (i, d).  Fuses the
// symmetrised -> primitive transform (dipole_kernals.cu:38-71) with the
// scatter of primitive roots onto their (key, J=0 index) position.
__global__ void k_build_y(const double* __restrict__ vecs, int ld, const int32_t* __restrict__ ivec,
                          int ndeg, const int32_t* __restrict__ yptr,
                          const int32_t* __restrict__ yroot, const int32_t* __restrict__ root_case,
                          const int32_t* __restrict__ root_lam,
                          const int32_t* __restrict__ case_iterm,
                          const int32_t* __restrict__ case_nelem, const double* __restrict__ rep,
                          int Ntot, int degen, int nslot, int N, int Kp, double* __restrict__ Y) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  const int col = blockIdx.y;  // i * ndeg + d
  const int i = col / ndeg, d = col - i * ndeg;
  if (e >= nslot * Kp) return;
  const int slot = e / Kp, v = e - slot * Kp;
  double acc = 0.0;
  if (v < N) {
    const double* vs = vecs + (size_t)ivec[i] * ld;
    const int q = slot * N + v;
    for (int p = yptr[q]; p < yptr[q + 1]; ++p) {
      const int r = yroot[p];
      const int c = root_case[r], lam = root_lam[r];
      const int it = case_iterm[c], ne = case_nelem[c];
      const double* rr = rep + (size_t)d * Ntot + (size_t)lam * degen * Ntot;
      for (int j = 0; j < ne; ++j) acc = fma(vs[it + j], rr[it + j], acc);
    }
  }
  Y[((size_t)col * nslot + slot) * Kp + v] = acc;
}

cudaError_t launch_build_y(const double* vecs, int ld, const int32_t* ivec, int nI, int ndeg,
                           const Basis& b, int gamma, int degen, int N, int Kp, double* Y,
                           cudaStream_t s, int d0) {
  if (nI == 0) return cudaSuccess;
  dim3 grid((b.nslot * Kp + 255) / 256, nI * ndeg);
  // d0: the first degenerate component (ndeg = 1, d0 = d: component d alone)
  k_build_y<<<grid, 256, 0, s>>>(vecs, ld, ivec, ndeg, b.d_yptr.p, b.d_yroot.p, b.d_root_case.p,
                                 b.d_root_lam.p, b.d_case_iterm[gamma].p,
                                 b.d_case_nelem[gamma].p,
                                 b.d_rep[gamma].p + (size_t)d0 * b.Ntotal[gamma], b.Ntotal[gamma],
                                 degen, b.nslot, N, Kp, Y);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ H build
// One thread per symmetrised final function s of one initial column (i, dI);
// writes H for every final degenerate component dF.
template <int NDEGF>
__device__ __forceinline__ void build_h_col(
    const double* __restrict__ Z, size_t zc, int ldz, int nslotI, int colI,
    const int32_t* __restrict__ s_case, const int32_t* __restrict__ case_ptr,
    const int32_t* __restrict__ case_roots, const int32_t* __restrict__ root_v,
    const int32_t* __restrict__ root_key, const int32_t* __restrict__ root_lam,
    const double* __restrict__ rep, int Ntot, const StencilTerm* __restrict__ st,
    const int32_t* __restrict__ st_n, int st_max, int nsizeF, int ldh, int s,
    double* __restrict__ H) {
  double acc[NDEGF];
#pragma unroll
  for (int d = 0; d < NDEGF; ++d) acc[d] = 0.0;
  if (s < nsizeF) {
    const double* zcol = Z + (size_t)colI * nslotI * ldz;
    const int cs = s_case[s];
    for (int p = case_ptr[cs]; p < case_ptr[cs + 1]; ++p) {
      const int r = case_roots[p];
      const int v = root_v[r], key = root_key[r], lam = root_lam[r];
      double h = 0.0;
      const int nt = st_n[key];
      for (int t = 0; t < nt; ++t) {
        const StencilTerm term = st[key * st_max + t];
        h = fma(term.coef, zcol[(size_t)term.c * zc + (size_t)term.slotI * ldz + v], h);
      }
#pragma unroll
      for (int d = 0; d < NDEGF; ++d)
        acc[d] = fma(rep[s + (size_t)d * Ntot + (size_t)lam * NDEGF * Ntot], h, acc[d]);
    }
  }
#pragma unroll
  for (int d = 0; d < NDEGF; ++d) H[((size_t)colI * NDEGF + d) * ldh + s] = acc[d];
}

template <int NDEGF>
__global__ void k_build_h(const double* __restrict__ Z, size_t zc, int ldz, int nslotI, int ndegI,
                          const int32_t* __restrict__ s_case, const int32_t* __restrict__ case_ptr,
                          const int32_t* __restrict__ case_roots,
                          const int32_t* __restrict__ root_v, const int32_t* __restrict__ root_key,
                          const int32_t* __restrict__ root_lam, const double* __restrict__ rep,
                          int Ntot, const StencilTerm* __restrict__ st,
                          const int32_t* __restrict__ st_n, int st_max, int nsizeF, int ldh,
                          double* __restrict__ H) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  const int colI = blockIdx.y;  // i * ndegI + dI
  if (s >= ldh) return;
  build_h_col<NDEGF>(Z, zc, ldz, nslotI, colI, s_case, case_ptr, case_roots, root_v, root_key,
                     root_lam, rep, Ntot, st, st_n, st_max, nsizeF, ldh, s, H);
}

// Every H build of a group of final blocks in one launch: item k covers
// blocks [items[k].blk0, items[k].blk0 + items[k].nblk) of the 1-D grid, each
// block 256 functions s of kHCols initial columns (the item lookup is paid
// once per kHCols columns).
__global__ void __launch_bounds__(256) k_build_h_items(const HItem* __restrict__ items,
                                                        const long long* __restrict__ firsts,
                                                        int nitems) {
  const long long b = blockIdx.x;
  const int lo = find_item(nitems, b, [&](int k) { return firsts[k]; });
  const HItem& it = items[lo];
  const long long rel = b - it.blk0;
  const int nsb = (it.ldh + 255) >> 8;
  const int cb = (int)(rel / nsb);
  const int s = (int)(rel - (long long)cb * nsb) * 256 + threadIdx.x;
  if (s >= it.ldh) return;
  const int c1 = min(it.ncol, (cb + 1) * kHCols);
  for (int colI = cb * kHCols; colI < c1; ++colI) {
    if (it.ndegF == 2)
      build_h_col<2>(it.Z, it.zc, it.ldz, it.nslotI, colI, it.s_case, it.case_ptr, it.case_roots,
                     it.root_v, it.root_key, it.root_lam, it.rep, it.Ntot, it.st, it.st_n,
                     it.st_max, it.nsizeF, it.ldh, s, it.H);
    else
      build_h_col<1>(it.Z, it.zc, it.ldz, it.nslotI, colI, it.s_case, it.case_ptr, it.case_roots,
                     it.root_v, it.root_key, it.root_lam, it.rep, it.Ntot, it.st, it.st_n,
                     it.st_max, it.nsizeF, it.ldh, s, it.H);
  }
}

cudaError_t launch_build_h_items(const HItem* items, const long long* firsts, int nitems,
                                 long long nblocks, cudaStream_t st) {
  if (nitems <= 0 || nblocks <= 0) return cudaSuccess;
  if (nblocks > 0x7FFFFFFFll) return cudaErrorInvalidValue;
  k_build_h_items<<<(unsigned)nblocks, 256, 0, st>>>(items, firsts, nitems);
  return cudaGetLastError();
}

// The item of an H build (one per (initial unit, final block) of a group).
HItem make_h_item(const double* Z, size_t zstride_c, int ldz, int nslotI, int ndegI, int nI,
                  const Basis& bF, int gammaF, int degF, int nsizeF, int ldh,
                  const StencilTerm* st, const int32_t* st_n, int st_max, double* H,
                  long long blk0) {
  HItem it{};
  it.Z = Z;
  it.zc = zstride_c;
  it.ldz = ldz;
  it.nslotI = nslotI;
  it.ndegF = degF;
  it.nsizeF = nsizeF;
  it.ldh = ldh;
  it.Ntot = bF.Ntotal[gammaF];
  it.st_max = st_max;
  it.s_case = bF.d_s_case[gammaF].p;
  it.case_ptr = bF.d_case_ptr.p;
  it.case_roots = bF.d_case_roots.p;
  it.root_v = bF.d_root_v.p;
  it.root_key = bF.d_root_key.p;
  it.root_lam = bF.d_root_lam.p;
  it.rep = bF.d_rep[gammaF].p;
  it.st = st;
  it.st_n = st_n;
  it.H = H;
  it.blk0 = blk0;
  it.ncol = nI * ndegI;
  it.nblk = (long long)((it.ncol + kHCols - 1) / kHCols) * ((ldh + 255) / 256);
  return it;
}

cudaError_t launch_build_h(const double* Z, size_t zstride_c, int ldz, int nslotI, int ndegI,
                           int nI, const Basis& bF, int gammaF, int degF, int nsizeF, int ldh,
                           const StencilTerm* st, const int32_t* st_n, int st_max, double* H,
                           cudaStream_t s) {
  if (nI == 0) return cudaSuccess;
  dim3 grid((ldh + 255) / 256, nI * ndegI);
  if (degF == 1)
    k_build_h<1><<<grid, 256, 0, s>>>(Z, zstride_c, ldz, nslotI, ndegI, bF.d_s_case[gammaF].p,
                                      bF.d_case_ptr.p, bF.d_case_roots.p, bF.d_root_v.p,
                                      bF.d_root_key.p, bF.d_root_lam.p, bF.d_rep[gammaF].p,
                                      bF.Ntotal[gammaF], st, st_n, st_max, nsizeF, ldh, H);
  else if (degF == 2)
    k_build_h<2><<<grid, 256, 0, s>>>(Z, zstride_c, ldz, nslotI, ndegI, bF.d_s_case[gammaF].p,
                                      bF.d_case_ptr.p, bF.d_case_roots.p, bF.d_root_v.p,
                                      bF.d_root_key.p, bF.d_root_lam.p, bF.d_rep[gammaF].p,
                                      bF.Ntotal[gammaF], st, st_n, st_max, nsizeF, ldh, H);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

// Primitive-space half line strength of one column (the reference's half_ls
// buffer, dipole_kernals.cu:223-224).
__global__ void k_half_ls_prim(const double* __restrict__ Z, size_t zc, int ldz,
                               const int32_t* __restrict__ root_v,
                               const int32_t* __restrict__ root_key,
                               const StencilTerm* __restrict__ st, const int32_t* __restrict__ st_n,
                               int st_max, int D, double* __restrict__ h) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= D) return;
  const int v = root_v[r], key = root_key[r];
  double acc = 0.0;
  for (int t = 0; t < st_n[key]; ++t) {
    const StencilTerm term = st[key * st_max + t];
    acc = fma(term.coef, Z[(size_t)term.c * zc + (size_t)term.slotI * ldz + v], acc);
  }
  h[r] = acc;
}

cudaError_t launch_half_ls_prim(const double* Z, size_t zstride_c, int ldz, const Basis& bF,
                                const StencilTerm* st, const int32_t* st_n, int st_max,
                                double* h, cudaStream_t s) {
  k_half_ls_prim<<<(bF.D + 255) / 256, 256, 0, s>>>(Z, zstride_c, ldz, bF.d_root_v.p,
                                                    bF.d_root_key.p, st, st_n, st_max, bF.D, h);
  return cudaGetLastError();
}

// The same from a Z split into K parts (the narrow split-precision GEMM):
// Z_c[col][v] = sum_p Zp[p][col][c * cstride + v], col = colbase + slot.
__global__ void k_half_ls_prim_parts(const double* __restrict__ Zp, int nparts, size_t pstride,
                                     int ldz, int cstride, const int32_t* __restrict__ root_v,
                                     const int32_t* __restrict__ root_key,
                                     const StencilTerm* __restrict__ st,
                                     const int32_t* __restrict__ st_n, int st_max, int D,
                                     double* __restrict__ h) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= D) return;
  const int v = root_v[r], key = root_key[r];
  double acc = 0.0;
  for (int t = 0; t < st_n[key]; ++t) {
    const StencilTerm term = st[key * st_max + t];
    const double* z = Zp + (size_t)term.slotI * ldz + (size_t)term.c * cstride + v;
    double zs = z[0];
    for (int p = 1; p < nparts; ++p) zs += z[(size_t)p * pstride];
    acc = fma(term.coef, zs, acc);
  }
  h[r] = acc;
}

cudaError_t launch_half_ls_prim_parts(const double* Zp, int nparts, size_t pstride, int ldz,
                                      int cstride, const Basis& bF, const StencilTerm* st,
                                      const int32_t* st_n, int st_max, double* h,
                                      cudaStream_t s) {
  k_half_ls_prim_parts<<<(bF.D + 255) / 256, 256, 0, s>>>(Zp, nparts, pstride, ldz, cstride,
                                                          bF.d_root_v.p, bF.d_root_key.p, st,
                                                          st_n, st_max, bF.D, h);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ epilogue
// One thread per (initial level i, final level f) of a part: the per-line
// epilogue of epilogue.cuh on the moments of T.
__global__ void k_epilogue(const double* __restrict__ T, int ldt, int nI, int nF,
                           const int32_t* __restrict__ levelI, const double* __restrict__ EI,
                           const int32_t* __restrict__ levelF, const double* __restrict__ EF,
                           const uint8_t* __restrict__ upper_ok,
                           const double* __restrict__ hn, EpiParams p,
                           gi_line* __restrict__ out, unsigned long long* counter,
                           long long cap, RefineRec* __restrict__ rec, long long rec_cap) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  const int i = blockIdx.y;
  // the initial level's Boltzmann factor, once per block (FP64 exp is scarce)
  __shared__ double boltz_i;
  if (threadIdx.x == 0) boltz_i = exp(-(EI[i] - p.zpe) * p.beta);
  __syncthreads();
  double t[4] = {0.0, 0.0, 0.0, 0.0}, hnq[4] = {0.0, 0.0, 0.0, 0.0};
  const bool ok_f = f < nF && upper_ok[f];
  if (ok_f)
    for (int dF = 0; dF < p.ndegF; ++dF)
      for (int dI = 0; dI < p.ndegI; ++dI)
        if (p.combo_mask & (1 << (dI + 2 * dF))) {
          const int col = (i * p.ndegI + dI) * p.ndegF + dF;
          t[dI + 2 * dF] = T[(size_t)col * ldt + f];
          hnq[dI + 2 * dF] = hn[col];
        }
  LineEval r;
  eval_line(p, t, hnq, EI[i], ok_f ? EF[f] : 0.0, boltz_i, ok_f, levelI[i],
            ok_f ? levelF[f] : -1, r);
  append_line(r, p.part, i, f, out, counter, cap, rec, rec_cap);
}

__global__ void k_boltz(const double* __restrict__ E, int n, double zpe, double beta,
                        double* __restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k < n) out[k] = exp(-(E[k] - zpe) * beta);
}

// Full line records -> compact ones (the read-back of GI_RUN_COMPACT_LINES).
__global__ void k_pack_lines(const gi_line* __restrict__ in, gi_line_compact* __restrict__ out,
                             long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const gi_line& L = in[i];
    gi_line_compact o;
    o.level_i = L.level_i;
    o.level_f = L.level_f;
    o.nu = L.nu;
    o.S = L.S;
    o.A = L.A;
    o.I = L.I;
    out[i] = o;
  }
}

cudaError_t launch_pack_lines(const gi_line* in, gi_line_compact* out, long long n,
                              cudaStream_t st) {
  if (n <= 0) return cudaSuccess;
  const long long blocks = std::min<long long>((n + 255) / 256, 152 * 16);
  k_pack_lines<<<(unsigned)blocks, 256, 0, st>>>(in, out, n);
  return cudaGetLastError();
}

cudaError_t launch_boltz(const double* E, int n, double zpe, double beta, double* out,
                         cudaStream_t s) {
  if (n <= 0) return cudaSuccess;
  k_boltz<<<(n + 255) / 256, 256, 0, s>>>(E, n, zpe, beta, out);
  return cudaGetLastError();
}

// Euclidean norm of each H column (the scale of its transition moments' error).
__global__ void k_col_norms(const double* __restrict__ H, int ldh, int n, double* __restrict__ out) {
  const double* h = H + (size_t)blockIdx.x * ldh;
  double acc = 0.0;
  for (int s = threadIdx.x; s < n; s += blockDim.x) acc = fma(h[s], h[s], acc);
  __shared__ double part[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) out[blockIdx.x] = sqrt(acc);
  }
}

// The columns of every H of a group in one launch (item k: columns
// [items[k].col0, items[k+1].col0) of the grid).
__global__ void k_col_norms_items(const NormItem* __restrict__ items, int nitems) {
  const long long b = blockIdx.x;
  const int lo = find_item(nitems, b, [&](int k) { return items[k].col0; });
  const NormItem& it = items[lo];
  const double* h = it.H + (size_t)(b - it.col0) * it.ldh;
  double acc = 0.0;
  for (int s = threadIdx.x; s < it.n; s += blockDim.x) acc = fma(h[s], h[s], acc);
  __shared__ double part[32];
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? part[threadIdx.x] : 0.0;
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if (threadIdx.x == 0) it.out[b - it.col0] = sqrt(acc);
  }
}

cudaError_t launch_col_norms_items(const NormItem* items, int nitems, long long ncol,
                                   cudaStream_t s) {
  if (nitems <= 0 || ncol <= 0) return cudaSuccess;
  if (ncol > 0x7FFFFFFFll) return cudaErrorInvalidValue;
  k_col_norms_items<<<(unsigned)ncol, 256, 0, s>>>(items, nitems);
  return cudaGetLastError();
}

cudaError_t launch_col_norms(const double* H, int ldh, int n, int ncol, double* out,
                             cudaStream_t s) {
  if (ncol <= 0) return cudaSuccess;
  k_col_norms<<<ncol, 256, 0, s>>>(H, ldh, n, out);
  return cudaGetLastError();
}

cudaError_t launch_epilogue(const double* T, int ldt, int nI, int nF, const int32_t* levelI,
                            const double* EI, const int32_t* levelF, const double* EF,
                            const uint8_t* upper_ok, const double* hn, const EpiParams& p,
                            gi_line* out, unsigned long long* counter, long long cap,
                            RefineRec* rec, long long rec_cap, cudaStream_t s) {
  if (nI == 0 || nF == 0) return cudaSuccess;
  dim3 grid((nF + 127) / 128, nI);
  k_epilogue<<<grid, 128, 0, s>>>(T, ldt, nI, nF, levelI, EI, levelF, EF, upper_ok, hn, p, out,
                                  counter, cap, rec, rec_cap);
  return cudaGetLastError();
}

// ------------------------------------------------------------------ FP64 GEMM
// C[z][n*ldc + m] = sum_k A[z][m*lda + k] * B[n*ldb + k] on the FP64 tensor
// pipe (mma.sync m8n8k4 .f64).  64x64 tile, 4 warps of 32x32, K step 16,
// cp.async double buffering.  K is a multiple of 16 and lda/ldb are even
// (the engine pads every K dimension), so each 16-byte copy is aligned.
namespace {
constexpr int GBM = 64, GBN = 64, GBK = 16, GPAD = 2;

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem, bool valid) {
  const unsigned sa = (unsigned)__cvta_generic_to_shared(smem);
  const int n = valid ? 16 : 0;
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(sa), "l"(gmem), "r"(n));
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N));
}
}  // namespace

__global__ void __launch_bounds__(128)
    k_gemm_fp64_nt(const double* __restrict__ A, int lda, size_t strideA,
                   const double* __restrict__ B, int ldb, double* __restrict__ C, int ldc,
                   size_t strideC, int M, int Nc, int K) {
  __shared__ __align__(16) double As[2][GBM][GBK + GPAD];
  __shared__ __align__(16) double Bs[2][GBN][GBK + GPAD];
  A += (size_t)blockIdx.z * strideA;
  C += (size_t)blockIdx.z * strideC;
  const int m0 = blockIdx.y * GBM, n0 = blockIdx.x * GBN;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, tq = lane & 3;

  double acc[4][4][2];
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b) acc[a][b][0] = acc[a][b][1] = 0.0;

  auto load = [&](int st, int k0) {
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int q = tid + 128 * j;
      const int row = q >> 3, cp = (q & 7) * 2;
      const int am = m0 + row, bn = n0 + row;
      const bool va = am < M, vb = bn < Nc;
      cp_async16(&As[st][row][cp], A + (size_t)(va ? am : 0) * lda + k0 + cp, va);
      cp_async16(&Bs[st][row][cp], B + (size_t)(vb ? bn : 0) * ldb + k0 + cp, vb);
    }
    cp_async_commit();
  };

  const int nk = K / GBK;
  load(0, 0);
  for (int kt = 0; kt < nk; ++kt) {
    const int st = kt & 1;
    if (kt + 1 < nk) {
      load(st ^ 1, (kt + 1) * GBK);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < GBK; kk += 4) {
      double af[4], bf[4];
#pragma unroll
      for (int a = 0; a < 4; ++a) af[a] = As[st][wm + a * 8 + g][kk + tq];
#pragma unroll
      for (int b = 0; b < 4; ++b) bf[b] = Bs[st][wn + b * 8 + g][kk + tq];
#pragma unroll
      for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b)
          asm volatile(
              "mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
              : "+d"(acc[a][b][0]), "+d"(acc[a][b][1])
              : "d"(af[a]), "d"(bf[b]));
    }
    __syncthreads();
  }
#pragma unroll
  for (int a = 0; a < 4; ++a)
#pragma unroll
    for (int b = 0; b < 4; ++b)
#pragma unroll
      for (int e = 0; e < 2; ++e) {
        const int m = m0 + wm + a * 8 + g;
        const int n = n0 + wn + b * 8 + tq * 2 + e;
        if (m < M && n < Nc) C[(size_t)n * ldc + m] = acc[a][b][e];
      }
}

cudaError_t gemm_fp64_nt(const double* A, int lda, size_t strideA, const double* B, int ldb,
                         double* C, int ldc, size_t strideC, int M, int Nc, int K, int batch,
                         cudaStream_t s) {
  if (M <= 0 || Nc <= 0 || batch <= 0) return cudaSuccess;
  if (K <= 0 || K % GBK != 0 || (lda & 1) || (ldb & 1)) return cudaErrorInvalidValue;
  dim3 grid((Nc + GBN - 1) / GBN, (M + GBM - 1) / GBM, batch);
  k_gemm_fp64_nt<<<grid, 128, 0, s>>>(A, lda, strideA, B, ldb, C, ldc, strideC, M, Nc, K);
  return cudaGetLastError();
}

}  // namespace gi
