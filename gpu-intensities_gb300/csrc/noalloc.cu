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
// every call because the scatter accumulates into it) and Z (3x that, fully
// written by the GEMM before it is read).  The 3j/K-tau term tables and the
// key -> slot map are device tables of the initial basis, built when the basis
// or the 3j table is set, so a call copies nothing from the host: it checks
// its arguments against sizes the setters recorded and enqueues device work.
// The array keeps the last call's contents; calls whose work overlaps on the
// GPU share the array and race, so a caller must order them (one stream, or
// events).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <mutex>

#include "engine.h"

namespace gi {
namespace {

constexpr int kMaxDevices = 64;
constexpr size_t kMaxElems = size_t(1) << 19;                     // ndeg * nslot * Kp of Y
constexpr size_t kScratchBytes = 4 * kMaxElems * sizeof(double);  // Y + 3 Z = 16 MiB
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
  if (elems > kMaxElems) {
    char buf[256];
    snprintf(buf, sizeof(buf),
             "gi_half_ls_noalloc: size beyond the fixed scratch: degen*slots*Kp = %zu > %zu "
             "(jI=%d); use gi_half_ls",
             elems, kMaxElems, jI);
    return say(GI_ERR_ARG, buf);
  }
  // every row index the kernels use must stay inside its Kp-wide row
  if (bI.iroot_max >= c->N || bF.iroot_max >= c->N)
    return say(GI_ERR_ARG, "gi_half_ls_noalloc: iroot_correlat_j0 >= N");
  const DevArray<StencilTerm>& d_st = bI.d_pair_st[jF - jI + 1];
  const DevArray<int32_t>& d_stn = bI.d_pair_stn[jF - jI + 1];
  if (!d_st.p || !d_stn.p || !bI.d_slot_of_key.p)
    return say(GI_ERR_STATE, "gi_half_ls_noalloc: the basis has no term tables");
  if (cudaSetDevice(c->device) != cudaSuccess)
    return say(GI_ERR_CUDA, "gi_half_ls_noalloc: cudaSetDevice failed");
  unsigned char* base = nullptr;
  if (scratch_address(c->device, &base) != cudaSuccess)
    return say(GI_ERR_CUDA, "gi_half_ls_noalloc: cudaGetSymbolAddress of the scratch failed");
  double* Y = reinterpret_cast<double*>(base);
  double* Z = Y + elems;
  cudaStream_t s = stream ? static_cast<cudaStream_t>(stream) : c->stream;

  cudaError_t e = cudaMemsetAsync(Y, 0, sizeof(double) * elems, s);
  if (e == cudaSuccess) {
    dim3 grid((bI.D + 255) / 256, ndeg);
    k_scatter_y<<<grid, 256, 0, s>>>(vsym_dev, bI.d_root_v.p, bI.d_root_key.p, bI.d_root_case.p,
                                     bI.d_root_lam.p, bI.d_case_iterm[gammaI].p,
                                     bI.d_case_nelem[gammaI].p, bI.d_rep[gammaI].p,
                                     bI.Ntotal[gammaI], ndeg, bI.d_slot_of_key.p, bI.D, bI.nslot,
                                     c->Kp, Y);
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
    e = launch_half_ls_prim(Z + (size_t)ideg * bI.nslot * c->Kp, zc, c->Kp, bF, d_st.p, d_stn.p,
                            6, half_ls_dev, s);
  if (e != cudaSuccess) {
    c->err = std::string("gi_half_ls_noalloc: ") + cudaGetErrorString(e);
    return GI_ERR_CUDA;
  }
  return GI_OK;
}
