// Allocation-free half line strength (gi_half_ls_noalloc in include/gi.h).
//
// Some callers of the per-vector half line strength cannot allocate device
// memory at the point where they call it: a serving loop whose HBM is fully
// reserved by its admission budget (a stray cudaMalloc could fail or push
// resident eigenvector blocks out), an upstream eigensolver or host framework
// that owns all device memory through its own pool and forbids other
// allocations, and latency-sensitive callers for whom cudaMalloc/cudaFree
// would add their implicit device-wide synchronisation to every call.  This
// entry point serves them: the caller passes device input and output buffers
// and the scratch lives in one file-scope device array of fixed size
// (kScratchBytes), which every GPU that loads the library holds until exit.
//
// Scratch use per call: Y (ndeg * nslot * Kp doubles, zeroed at the start of
// every call because the scatter accumulates into it), Z (3x that, fully
// written by the GEMM before it is read), the 3j/K-tau term table and the
// key -> slot map (both copied in at the start of every call).  The array
// keeps the last call's contents; calls whose work overlaps on the GPU share
// the array and race, so a caller must order them (one stream, or events).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "engine.h"

namespace gi {
namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kMaxElems = size_t(1) << 19;      // ndeg * nslot * Kp of Y
constexpr int kMaxKeys = 512;                      // 2*J+2 for J <= 255
constexpr size_t kYZBytes = 4 * kMaxElems * sizeof(double);  // Y + 3 Z = 16 MiB
constexpr size_t kStencilBytes = (size_t)kMaxKeys * 6 * sizeof(StencilTerm);
constexpr size_t kScratchBytes = kYZBytes + kStencilBytes + 2 * kMaxKeys * sizeof(int32_t);
static_assert(kScratchBytes == GI_NOALLOC_SCRATCH_BYTES, "scratch size stated in gi.h");

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mutex;
void* g_scratch_dev[kMaxDevices] = {};

// Device address of the scratch array on `device`, looked up once per device
// with that device current.  In host code the array's name is only a
// host-side stand-in, so kernels must be given this address.
cudaError_t scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mutex);
  if (!g_scratch_dev[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch_dev[device] = p;
  }
  *out = static_cast<unsigned char*>(g_scratch_dev[device]);
  return cudaSuccess;
}

// Symmetrised -> primitive transform of one initial vector (the arithmetic of
// k_build_y, dipole_kernals.cu:38-71), scattered onto Y[d][slot][v] with an
// atomic add so that no (slot, v) index table is needed.
__global__ void k_scatter_y(const double* __restrict__ vsym, const int32_t* __restrict__ root_v,
                            const int32_t* __restrict__ root_key,
                            const int32_t* __restrict__ root_case,
                            const int32_t* __restrict__ root_lam,
                            const int32_t* __restrict__ case_iterm,
                            const int32_t* __restrict__ case_nelem,
                            const double* __restrict__ rep, int Ntot, int degen,
                            const int32_t* __restrict__ slot_of_key, int D, int nslot, int Kp,
                            double* __restrict__ Y) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  const int d = blockIdx.y;
  if (r >= D) return;
  const int c = root_case[r], lam = root_lam[r];
  const int it = case_iterm[c], ne = case_nelem[c];
  const double* rr = rep + (size_t)d * Ntot + (size_t)lam * degen * Ntot;
  double acc = 0.0;
  for (int j = 0; j < ne; ++j) acc = fma(vsym[it + j], rr[it + j], acc);
  const int slot = slot_of_key[root_key[r]];
  atomicAdd(&Y[((size_t)d * nslot + slot) * Kp + root_v[r]], acc);
}

}  // namespace
}  // namespace gi

using namespace gi;

extern "C" gi_status gi_half_ls_noalloc(gi_ctx* h, int jI, int gammaI, int ideg, int jF,
                                        const double* vsym_dev, double* half_ls_dev,
                                        void* stream) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !vsym_dev || !half_ls_dev) return GI_ERR_ARG;
  auto say = [c](gi_status s, const char* msg) {
    c->err = msg;
    return s;
  };
  if (c->N == 0) return say(GI_ERR_STATE, "gi_half_ls_noalloc: gi_set_dipole not called");
  auto iI = c->bases.find(jI), iF = c->bases.find(jF);
  if (iI == c->bases.end() || iF == c->bases.end())
    return say(GI_ERR_NOTFOUND, "gi_half_ls_noalloc: no basis for jI or jF");
  if (gammaI < 0 || gammaI >= c->nrep || ideg < 0 || ideg >= c->degen[gammaI])
    return say(GI_ERR_ARG, "gi_half_ls_noalloc: bad gammaI or ideg");
  if (std::abs(jI - jF) > 1) return say(GI_ERR_ARG, "gi_half_ls_noalloc: |jI - jF| > 1");
  const Basis& bI = *iI->second;
  const Basis& bF = *iF->second;
  const int ndeg = c->degen[gammaI];
  const size_t elems = (size_t)ndeg * bI.nslot * c->Kp;
  if (elems > kMaxElems || 2 * jI + 2 > kMaxKeys || 2 * jF + 2 > kMaxKeys) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "gi_half_ls_noalloc: size beyond the fixed scratch: degen*slots*Kp = %zu > %zu, or "
             "J > %d (jI=%d, jF=%d); use gi_half_ls",
             elems, kMaxElems, kMaxKeys / 2 - 1, jI, jF);
    return say(GI_ERR_ARG, buf);
  }
  // every row index the kernels use must stay inside its Kp-wide row
  for (int r = 0; r < bI.D; r++)
    if (bI.iroot[r] >= c->N) return say(GI_ERR_ARG, "gi_half_ls_noalloc: iroot_correlat_j0 >= N");
  for (int r = 0; r < bF.D; r++)
    if (bF.iroot[r] >= c->N) return say(GI_ERR_ARG, "gi_half_ls_noalloc: iroot_correlat_j0 >= N");
  if (cudaSetDevice(c->device) != cudaSuccess)
    return say(GI_ERR_CUDA, "gi_half_ls_noalloc: cudaSetDevice failed");
  unsigned char* base = nullptr;
  if (scratch_address(c->device, &base) != cudaSuccess)
    return say(GI_ERR_CUDA, "gi_half_ls_noalloc: cudaGetSymbolAddress of the scratch failed");
  double* Y = reinterpret_cast<double*>(base);
  double* Z = Y + elems;
  StencilTerm* d_st = reinterpret_cast<StencilTerm*>(base + kYZBytes);
  int32_t* d_stn = reinterpret_cast<int32_t*>(base + kYZBytes + kStencilBytes);
  int32_t* d_slot = d_stn + kMaxKeys;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;

  // host-side tables on the stack; a copy from pageable memory returns once
  // the source has been staged, so they may go out of scope afterwards
  StencilTerm st[kMaxKeys * 6];
  int32_t stn[kMaxKeys];
  int32_t slot_of_key[kMaxKeys];
  const bool table = c->threej_jmax >= std::max(jI, jF) && !c->threej.empty();
  stencil_fill(bI, bF, table ? c->threej.data() : nullptr, c->threej_jmax, st, stn);
  const int nkeyI = 2 * jI + 2, nkeyF = 2 * jF + 2;
  for (int k = 0; k < nkeyI; k++) slot_of_key[k] = bI.slot_of_key[k];

  cudaError_t e = cudaMemsetAsync(Y, 0, sizeof(double) * elems, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_st, st, sizeof(StencilTerm) * nkeyF * 6, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_stn, stn, sizeof(int32_t) * nkeyF, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(d_slot, slot_of_key, sizeof(int32_t) * nkeyI, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) {
    dim3 grid((bI.D + 255) / 256, ndeg);
    k_scatter_y<<<grid, 256, 0, s>>>(vsym_dev, bI.d_root_v.p, bI.d_root_key.p, bI.d_root_case.p,
                                     bI.d_root_lam.p, bI.d_case_iterm[gammaI].p,
                                     bI.d_case_nelem[gammaI].p, bI.d_rep[gammaI].p,
                                     bI.Ntotal[gammaI], ndeg, d_slot, bI.D, bI.nslot, c->Kp, Y);
    e = cudaGetLastError();
  }
  const int ncol = ndeg * bI.nslot;
  const size_t zc = (size_t)ncol * c->Kp;
  if (e == cudaSuccess) {
    // a streamed dipole passes through its preallocated staging panels
    const gi_status g = for_each_dipole_panel(c, s, [&](const double* mu, size_t ms, int rows,
                                                         int f0) {
      e = gemm_fp64_nt(mu, c->Kp, ms, Y, c->Kp, Z + f0, c->Kp, zc, rows, ncol, c->Kp, 3, s);
      return e == cudaSuccess ? GI_OK : GI_ERR_CUDA;
    });
    if (g != GI_OK && e == cudaSuccess) return g;  // a stream/event call failed (c->err set)
  }
  if (e == cudaSuccess)
    e = launch_half_ls_prim(Z + (size_t)ideg * bI.nslot * c->Kp, zc, c->Kp, bF, d_st, d_stn, 6,
                            half_ls_dev, s);
  if (e != cudaSuccess) {
    c->err = std::string("gi_half_ls_noalloc: ") + cudaGetErrorString(e);
    return GI_ERR_CUDA;
  }
  return GI_OK;
}
