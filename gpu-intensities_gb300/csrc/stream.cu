// A dipole that stays in host memory, streamed through the device in panels
// (gi_set_dipole_streamed in include/gi.h).
//
// The reference splits a dipole above 5 GiB into F-column blocks held on the
// host (read_dipole_flipped_blocks, trove_functions.cpp:207-310) and, for
// every initial vector, copies each block to the device and runs the
// half-line-strength kernel over its F range (do_1st_half_ls_blocks,
// cuda_host.cu:783-817).  Here a panel is a range [f0, f0 + rows) of rows f of
// all three components ([3][rows][Kp] on the device, the resident layout's
// rows), and one pass over the panels serves a whole round of initial levels:
// the half-ls GEMM Z_c = mu_c^T Y produces rows f of Z independently, so the
// GEMM of panel p writes Z rows [f0, f0 + rows) with the same per-element
// reduction as the resident GEMM (bit-identical).  Two staging panels on the
// device and a copy stream overlap the copy of panel p+1 with the
// contraction of panel p:
//
//   copy stream:    wait consumed[b]; H2D panel -> stage[b]; record loaded[b]
//   compute stream: wait loaded[b]; contraction of stage[b]; record consumed[b]
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>

#include "engine.h"
#include "split.h"

namespace gi {

struct DipoleStream {
  int N = 0, Kp = 0, panel = 0;
  double* host = nullptr;     // [3][N][N] record order (rows f)
  bool owned = false;         // host is the engine's pinned copy
  bool registered = false;    // host is the caller's array, page-locked here
  DevArray<double> stage[2];  // [3][panel][Kp], padding columns zero
  cudaStream_t copy = nullptr;
  cudaEvent_t loaded[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
  ~DipoleStream() {
    if (copy) cudaStreamSynchronize(copy);
    for (int b = 0; b < 2; b++) {
      if (loaded[b]) cudaEventDestroy(loaded[b]);
      if (consumed[b]) cudaEventDestroy(consumed[b]);
    }
    if (copy) cudaStreamDestroy(copy);
    if (owned) cudaFreeHost(host);
    if (registered) cudaHostUnregister(host);
  }
};

namespace {

// Rows per panel for about `bytes` of staging (two [3][rows][Kp] panels plus,
// on the split path, the panel's digits: 9 bf16 planes at most).
int auto_panel_rows(int N, int Kp) {
  const double per_row = (2.0 * 3 * 8 + 3.0 * 9 * 2) * Kp;
  const double rows = (double)GI_DIPOLE_PANEL_BYTES / per_row;
  int p = (int)std::min<double>(rows, N);
  if (p >= 128 && p < N) p -= p % 128;  // whole 128-row tiles except the last panel
  return std::max(p, 1);
}

gi_status install(Ctx* c, int N, double* host, bool owned, bool registered, int panel_rows) {
  const int Kp = round_up(N, 64);
  DipoleStream* d = new DipoleStream();
  d->N = N;
  d->Kp = Kp;
  d->host = host;
  d->owned = owned;
  d->registered = registered;
  d->panel = panel_rows > 0 ? std::min(panel_rows, N) : auto_panel_rows(N, Kp);
  const size_t elems = (size_t)3 * d->panel * Kp;
  cudaError_t e = cudaSuccess;
  for (int b = 0; b < 2 && e == cudaSuccess; b++) {
    e = d->stage[b].alloc(elems);
    if (e == cudaSuccess) e = cudaMemset(d->stage[b].p, 0, sizeof(double) * elems);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d->loaded[b], cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&d->consumed[b], cudaEventDisableTiming);
  }
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&d->copy, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaDeviceSynchronize();  // zero padding before any copy
  if (e != cudaSuccess) {
    d->owned = d->registered = false;  // the host array stays the caller's to release
    delete d;
    return fail(c, e == cudaErrorMemoryAllocation ? GI_ERR_NOMEM : GI_ERR_CUDA,
                "streamed dipole staging: %s", cudaGetErrorString(e));
  }
  dipole_stream_release(c);
  c->d_mu.reset();  // the resident copy, if any, is replaced
  c->dstream = d;
  c->N = N;
  c->Kp = Kp;
  split_invalidate(c);
  return GI_OK;
}

}  // namespace

void dipole_stream_release(Ctx* c) {
  delete c->dstream;
  c->dstream = nullptr;
}

int dipole_panel_rows(const Ctx* c) {
  const DipoleStream* d = c->parent ? c->parent->dstream : c->dstream;
  return d ? d->panel : 0;
}

gi_status dipole_stream_adopt(Ctx* c, int N, double* pinned, int panel_rows) {
  cudaSetDevice(c->device);
  gi_status s = install(c, N, pinned, /*owned=*/true, false, panel_rows);
  if (s != GI_OK) cudaFreeHost(pinned);
  return s;
}

gi_status for_each_dipole_panel(Ctx* c, cudaStream_t st, const PanelFn& fn) {
  DipoleStream* d = c->parent ? c->parent->dstream : c->dstream;
  if (!d) return fn(c->mu(), (size_t)c->N * c->Kp, c->N, 0);
  const int N = d->N, P = d->panel, Kp = d->Kp;
  const int npanel = (N + P - 1) / P;
  auto issue_copy = [&](int p) -> gi_status {
    const int b = p & 1, f0 = p * P, rows = std::min(P, N - f0);
    GI_CUDA(c, cudaStreamWaitEvent(d->copy, d->consumed[b], 0));
    for (int comp = 0; comp < 3; comp++)
      GI_CUDA(c, cudaMemcpy2DAsync(d->stage[b].p + (size_t)comp * P * Kp, sizeof(double) * Kp,
                                   d->host + (size_t)comp * N * N + (size_t)f0 * N,
                                   sizeof(double) * N, sizeof(double) * N, rows,
                                   cudaMemcpyHostToDevice, d->copy));
    GI_CUDA(c, cudaEventRecord(d->loaded[b], d->copy));
    return GI_OK;
  };
  // consumed[b] was last recorded after the previous contraction that read
  // stage[b] (on whichever stream): no copy overwrites a panel in use
  gi_status s = issue_copy(0);
  for (int p = 0; p < npanel && s == GI_OK; p++) {
    const int b = p & 1, f0 = p * P, rows = std::min(P, N - f0);
    if (p + 1 < npanel) s = issue_copy(p + 1);
    if (s != GI_OK) break;
    GI_CUDA(c, cudaStreamWaitEvent(st, d->loaded[b], 0));
    s = fn(d->stage[b].p, (size_t)P * Kp, rows, f0);
    if (s != GI_OK) break;
    GI_CUDA(c, cudaEventRecord(d->consumed[b], st));
  }
  return s;
}

gi_status dipole_gemm_fp64(Ctx* c, const double* Y, int ldy, double* Z, int ldz, size_t zc,
                           int ncol, cudaStream_t st) {
  return for_each_dipole_panel(c, st, [&](const double* mu, size_t mstride, int rows, int f0) {
    GI_CUDA(c, timed(c, GI_PHASE_HALFLS_GEMM, [&] {
              return gemm_fp64_nt(mu, c->Kp, mstride, Y, ldy, Z + f0, ldz, zc, rows, ncol, c->Kp,
                                  3, st);
            }));
    return GI_OK;
  });
}

}  // namespace gi

extern "C" {

gi_status gi_set_dipole_streamed(gi_ctx* h, int N, const double* mu, int panel_rows, int flags) {
  using namespace gi;
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || N <= 0 || !mu || panel_rows < 0 || (flags & ~GI_DIPOLE_BORROW)) return GI_ERR_ARG;
  if (c->server) return fail(c, GI_ERR_STATE, "gi_set_dipole_streamed while serving");
  cudaSetDevice(c->device);
  const size_t bytes = sizeof(double) * 3 * (size_t)N * N;
  double* host = const_cast<double*>(mu);
  if (flags & GI_DIPOLE_BORROW) {
    cudaError_t e = cudaHostRegister(host, bytes, cudaHostRegisterReadOnly);
    if (e != cudaSuccess && e != cudaErrorHostMemoryAlreadyRegistered) {
      cudaGetLastError();  // read-only registration is optional: plain page-locking
      e = cudaHostRegister(host, bytes, cudaHostRegisterDefault);
    }
    bool registered = true;
    if (e == cudaErrorHostMemoryAlreadyRegistered) {  // already page-locked by the caller
      cudaGetLastError();
      registered = false;
    } else if (e != cudaSuccess) {
      cudaGetLastError();
      return fail(c, GI_ERR_CUDA, "gi_set_dipole_streamed: cannot page-lock the dipole: %s",
                  cudaGetErrorString(e));
    }
    gi_status s = install(c, N, host, false, registered, panel_rows);
    if (s != GI_OK && registered) cudaHostUnregister(host);
    return s;
  }
  double* pinned = nullptr;
  GI_CUDA(c, cudaMallocHost(&pinned, bytes));
  std::memcpy(pinned, mu, bytes);
  return dipole_stream_adopt(c, N, pinned, panel_rows);
}

int gi_dipole_panel_rows(const gi_ctx* h) {
  const gi::Ctx* c = reinterpret_cast<const gi::Ctx*>(h);
  return c ? gi::dipole_panel_rows(c) : 0;
}

}  // extern "C"
