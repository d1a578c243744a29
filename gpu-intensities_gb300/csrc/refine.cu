// Exact re-evaluation of doubtful lines.
//
// The GEMM paths give each transition moment t an error of a few units of
// FP64 rounding of its column's norm (the half line strength Z = mu^T Y and
// the final contraction both round in FP64 or truncate digit planes there).
// Two kinds of line cannot carry that error:
//   * lines whose S or I sits within it of a threshold: the keep decision of
//     the reference's filter (cuda_host.cu:1408, applied here) would depend on
//     rounding;
//   * lines whose moment cancels far below its terms, where that error is a
//     large fraction of t (asked for when the context's refine limit is > 0).
// The epilogue hands such lines over (RefineRec).  For every initial column
// they touch, this file recomputes the column in double-double arithmetic on
// the CUDA cores: the symmetrised -> primitive transform and the scatter onto
// (key, J=0 index) (dipole_kernals.cu:38-71), Z = mu^T Y, the 3j/K-tau
// stencil (dipole_kernals.cu:162-227), the final vector's transform and the
// final dot (cuda_host.cu:1301-1317), each product formed exactly (TwoProd)
// and each sum carried as a (hi, lo) pair.  Then S, A and I are formed in FP64
// as the epilogue forms them (cuda_host.cu:1388-1407), the keep decision is
// taken again, and the line list is patched.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <map>
#include <tuple>
#include <vector>

#include "engine.h"

namespace gi {
namespace {

struct dd {
  double hi, lo;
};
__device__ __forceinline__ dd dd_norm(double s, double e) {
  const double h = s + e;
  return dd{h, e - (h - s)};
}
__device__ __forceinline__ dd dd_add(dd a, dd b) {
  const double s = a.hi + b.hi;
  const double z = s - a.hi;
  const double e = (a.hi - (s - z)) + (b.hi - z) + a.lo + b.lo;
  return dd_norm(s, e);
}
// acc + x * y with x exact in FP64 and y = (hi, lo)
__device__ __forceinline__ dd dd_fma1(dd acc, double x, dd y) {
  const double p = x * y.hi;
  const double pe = fma(x, y.hi, -p) + x * y.lo;
  return dd_add(acc, dd{p, pe});
}
// acc + x * y, both (hi, lo)
__device__ __forceinline__ dd dd_fma2(dd acc, dd x, dd y) {
  const double p = x.hi * y.hi;
  const double pe = fma(x.hi, y.hi, -p) + (x.hi * y.lo + x.lo * y.hi);
  return dd_add(acc, dd{p, pe});
}
__device__ __forceinline__ dd dd_shfl_down(dd v, int o) {
  return dd{__shfl_down_sync(0xffffffffu, v.hi, o), __shfl_down_sync(0xffffffffu, v.lo, o)};
}

// Y[slot][v] of one initial column (vector row vs, component d), double-double.
__global__ void k_dd_y(const double* __restrict__ vs, int d, const int32_t* __restrict__ yptr,
                       const int32_t* __restrict__ yroot, const int32_t* __restrict__ root_case,
                       const int32_t* __restrict__ root_lam,
                       const int32_t* __restrict__ case_iterm,
                       const int32_t* __restrict__ case_nelem, const double* __restrict__ rep,
                       int Ntot, int degen, int nslot, int N, double* __restrict__ Yh,
                       double* __restrict__ Yl) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= nslot * N) return;
  dd acc{0.0, 0.0};
  for (int p = yptr[e]; p < yptr[e + 1]; ++p) {
    const int r = yroot[p];
    const int c = root_case[r], lam = root_lam[r];
    const int it = case_iterm[c], ne = case_nelem[c];
    const double* rr = rep + (size_t)d * Ntot + (size_t)lam * degen * Ntot;
    for (int j = 0; j < ne; ++j) acc = dd_fma1(acc, vs[it + j], dd{rr[it + j], 0.0});
  }
  Yh[e] = acc.hi;
  Yl[e] = acc.lo;
}

// Z_c[slot][f] = sum_v mu_c(v, f) Y[slot][v] for rows f of one dipole panel:
// one warp per (c, slot, f), lanes along v, a double-double warp sum.
__global__ void k_dd_z(const double* __restrict__ mu, size_t mstride, int Kp, int rows, int f0,
                       const double* __restrict__ Yh, const double* __restrict__ Yl, int nslot,
                       int N, double* __restrict__ Zh, double* __restrict__ Zl) {
  const int wid = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (wid >= 3 * nslot * rows) return;
  const int fr = wid % rows, cs = wid / rows;
  const int slot = cs % nslot, c = cs / nslot;
  const double* m = mu + (size_t)c * mstride + (size_t)fr * Kp;
  const double* yh = Yh + (size_t)slot * N;
  const double* yl = Yl + (size_t)slot * N;
  dd acc{0.0, 0.0};
  for (int v = lane; v < N; v += 32) acc = dd_fma1(acc, m[v], dd{yh[v], yl[v]});
  for (int o = 16; o > 0; o >>= 1) acc = dd_add(acc, dd_shfl_down(acc, o));
  if (lane == 0) {
    const size_t o = ((size_t)c * nslot + slot) * N + f0 + fr;
    Zh[o] = acc.hi;
    Zl[o] = acc.lo;
  }
}

// One transition moment per block: t = sum_rF corrF[rF] h[rF] with
// h[rF] = sum_terms coef Z_c[slot][v(rF)] and corrF the final vector's
// primitive form (component dF), all in double-double.
struct TJob {
  const double* vf;  // final vector row
  int dF;
  int out;           // index into the result array
};
__global__ void k_dd_t(const TJob* __restrict__ jobs, const double* __restrict__ Zh,
                       const double* __restrict__ Zl, int nslotI, int N,
                       const int32_t* __restrict__ root_v, const int32_t* __restrict__ root_key,
                       const int32_t* __restrict__ root_case, const int32_t* __restrict__ root_lam,
                       const int32_t* __restrict__ case_iterm,
                       const int32_t* __restrict__ case_nelem, const double* __restrict__ rep,
                       int Ntot, int degen, const StencilTerm* __restrict__ st,
                       const int32_t* __restrict__ st_n, int D, double* __restrict__ out) {
  const TJob jb = jobs[blockIdx.x];
  dd acc{0.0, 0.0};
  for (int r = threadIdx.x; r < D; r += blockDim.x) {
    const int v = root_v[r], key = root_key[r];
    dd h{0.0, 0.0};
    for (int t = 0; t < st_n[key]; ++t) {
      const StencilTerm term = st[key * 6 + t];
      const size_t o = ((size_t)term.c * nslotI + term.slotI) * N + v;
      h = dd_fma1(h, term.coef, dd{Zh[o], Zl[o]});
    }
    const int c = root_case[r], lam = root_lam[r];
    const int it = case_iterm[c], ne = case_nelem[c];
    const double* rr = rep + (size_t)jb.dF * Ntot + (size_t)lam * degen * Ntot;
    dd cf{0.0, 0.0};
    for (int j = 0; j < ne; ++j) cf = dd_fma1(cf, jb.vf[it + j], dd{rr[it + j], 0.0});
    acc = dd_fma2(acc, cf, h);
  }
  for (int o = 16; o > 0; o >>= 1) acc = dd_add(acc, dd_shfl_down(acc, o));
  __shared__ double sh[32], sl[32];
  const int w = threadIdx.x >> 5;
  if ((threadIdx.x & 31) == 0) {
    sh[w] = acc.hi;
    sl[w] = acc.lo;
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    acc = threadIdx.x < (blockDim.x >> 5) ? dd{sh[threadIdx.x], sl[threadIdx.x]} : dd{0.0, 0.0};
    for (int o = 16; o > 0; o >>= 1) acc = dd_add(acc, dd_shfl_down(acc, o));
    if (threadIdx.x == 0) out[jb.out] = acc.hi + acc.lo;
  }
}

}  // namespace

gi_status refine_lines(Ctx* c, const std::vector<RefinePart>& parts, const RefineRec* recs,
                       size_t n, int64_t* refined) {
  *refined = 0;
  if (n == 0) return GI_OK;
  cudaStream_t st = c->stream;
  // group the records by initial column: (part, i); every record needs the
  // columns of all its initial components
  std::map<std::pair<int, int>, std::vector<size_t>> groups;
  for (size_t k = 0; k < n; k++) {
    if (recs[k].part < 0 || recs[k].part >= (int)parts.size())
      return fail(c, GI_ERR_DEVICE, "refinement record of an unknown part");
    groups[{recs[k].part, recs[k].i}].push_back(k);
  }
  std::vector<double> tvals(n * 4, 0.0);
  DevArray<double> yh, yl, zh, zl, tout;
  DevArray<TJob> djobs;
  for (auto& g : groups) {
    const RefinePart& P = parts[g.first.first];
    const int i = g.first.second;
    const Basis& bI = *P.basI;
    const Basis& bF = *P.basF;
    const int N = c->N, nslot = bI.nslot;
    const int ndegI = P.ep.ndegI, ndegF = P.ep.ndegF;
    const double* vi = P.bI->d_vecs.p + (size_t)P.rec_i[i] * P.bI->ld;
    GI_CUDA(c, yh.reserve((size_t)nslot * N));
    GI_CUDA(c, yl.reserve((size_t)nslot * N));
    GI_CUDA(c, zh.reserve((size_t)3 * nslot * N * ndegI));
    GI_CUDA(c, zl.reserve((size_t)3 * nslot * N * ndegI));
    const size_t zsz = (size_t)3 * nslot * N;
    for (int dI = 0; dI < ndegI; dI++) {
      k_dd_y<<<(nslot * N + 255) / 256, 256, 0, st>>>(
          vi, dI, bI.d_yptr.p, bI.d_yroot.p, bI.d_root_case.p, bI.d_root_lam.p,
          bI.d_case_iterm[P.gI].p, bI.d_case_nelem[P.gI].p, bI.d_rep[P.gI].p, bI.Ntotal[P.gI],
          ndegI, nslot, N, yh.p, yl.p);
      GI_CUDA(c, cudaGetLastError());
      double* Zh = zh.p + dI * zsz;
      double* Zl = zl.p + dI * zsz;
      gi_status s = for_each_dipole_panel(c, st, [&](const double* mu, size_t ms, int rows,
                                                     int f0) -> gi_status {
        const long long warps = 3LL * nslot * rows;
        k_dd_z<<<(unsigned)((warps + 7) / 8), 256, 0, st>>>(mu, ms, c->Kp, rows, f0, yh.p, yl.p,
                                                            nslot, N, Zh, Zl);
        GI_CUDA(c, cudaGetLastError());
        return GI_OK;
      });
      if (s != GI_OK) return s;
    }
    // one block per (record, combination of degenerate components), the jobs
    // of one initial component contiguous (they share its Z)
    std::vector<TJob> jobs;
    std::vector<size_t> first(ndegI + 1, 0);
    for (int dI = 0; dI < ndegI; dI++) {
      first[dI] = jobs.size();
      for (size_t k : g.second) {
        const double* vf = P.bF->d_vecs.p + (size_t)recs[k].f * P.bF->ld;
        for (int dF = 0; dF < ndegF; dF++)
          if (P.ep.combo_mask & (1 << (dI + 2 * dF)))
            jobs.push_back(TJob{vf, dF, (int)(k * 4 + dI + 2 * dF)});
      }
    }
    first[ndegI] = jobs.size();
    if (jobs.empty()) continue;
    GI_CUDA(c, djobs.reserve(jobs.size()));
    GI_CUDA(c, tout.reserve(n * 4));
    GI_CUDA(c, cudaMemcpyAsync(djobs.p, jobs.data(), sizeof(TJob) * jobs.size(),
                               cudaMemcpyHostToDevice, st));
    for (int dI = 0; dI < ndegI; dI++) {
      const size_t nj = first[dI + 1] - first[dI];
      if (nj == 0) continue;
      k_dd_t<<<(unsigned)nj, 256, 0, st>>>(
          djobs.p + first[dI], zh.p + dI * zsz, zl.p + dI * zsz, nslot, N, bF.d_root_v.p,
          bF.d_root_key.p, bF.d_root_case.p, bF.d_root_lam.p, bF.d_case_iterm[P.gF].p,
          bF.d_case_nelem[P.gF].p, bF.d_rep[P.gF].p, bF.Ntotal[P.gF], ndegF, P.st_dev,
          P.stn_dev, bF.D, tout.p);
      GI_CUDA(c, cudaGetLastError());
    }
    // the job arrays and Z are reused by the next group: finish this one
    GI_CUDA(c, cudaStreamSynchronize(st));
  }
  if (tout.p)
    GI_CUDA(c, cudaMemcpy(tvals.data(), tout.p, sizeof(double) * n * 4, cudaMemcpyDeviceToHost));

  // S, A, I and the keep decision in FP64, formed as the epilogue forms them
  std::vector<gi_line> upd;        // lines that stay, new values
  std::vector<int64_t> upd_slot;
  std::vector<gi_line> add;        // lines that now pass the thresholds
  std::vector<int64_t> drop;       // slots of lines that no longer pass
  for (size_t k = 0; k < n; k++) {
    const RefineRec& R = recs[k];
    const RefinePart& P = parts[R.part];
    const EpiParams& p = P.ep;
    double t[4] = {0.0, 0.0, 0.0, 0.0};
    for (int dF = 0; dF < p.ndegF; ++dF)
      for (int dI = 0; dI < p.ndegI; ++dI)
        if (p.combo_mask & (1 << (dI + 2 * dF))) t[dI + 2 * dF] = tvals[k * 4 + dI + 2 * dF];
    double ls = 0.0;
    for (int dF = 0; dF < p.ndegF; ++dF)
      for (int dI = 0; dI < p.ndegI; ++dI) ls += t[dI + 2 * dF] * t[dI + 2 * dF];
    ls /= (double)p.ndegI;
    if (p.reduced && p.ndegF != 1 && p.ndegI != 1) ls *= (double)p.ndegI;
    const double ei = P.EI[R.i], ef = P.bF->energies[R.f];
    const double nu = ef - ei;
    const double anu = std::fabs(nu);
    const double boltz_i = std::exp(-(ei - p.zpe) * p.beta);
    const double boltz_fc = anu * boltz_i * (1.0 - std::exp(-anu * p.beta)) / p.q_stat;
    gi_line L{};
    L.level_i = P.lvl_i[R.i];
    L.level_f = P.lvl_f[R.f];
    L.ndeg_i = p.ndegI;
    L.ndeg_f = p.ndegF;
    L.nu = nu;
    L.A = p.A_coef * (double)(2 * p.jI + 1) * ls * (anu * anu * anu);
    L.S = ls * p.gns * (double)((2 * p.jI + 1) * (2 * p.jF + 1));
    L.I = L.S * p.intens_cm_mol * boltz_fc;
    for (int q = 0; q < 4; ++q) L.t[q] = t[q];
    const bool keep = (L.S >= p.thresh_S) && (L.I / p.avogno >= p.thresh_I);
    if (R.slot >= 0 && keep) {
      upd.push_back(L);
      upd_slot.push_back(R.slot);
    } else if (R.slot >= 0) {
      drop.push_back(R.slot);
    } else if (keep) {
      add.push_back(L);
    }
  }

  // patch the line list (device, and the host copy when the lines went there)
  const bool host = !c->lines_on_device;
  gi_line* d = c->d_lines.p;
  int64_t count = c->nlines;
  const int64_t need = count + (int64_t)add.size();
  if ((size_t)need > c->d_lines.n)
    return fail(c, GI_ERR_DEVICE, "line buffer overflow after refinement");
  const bool compact = host && c->compact_lines;  // the host holds compact records
  if (compact && c->h_compact_cap < (size_t)need) {
    gi_line_compact* nh = nullptr;
    GI_CUDA(c, cudaMallocHost(reinterpret_cast<void**>(&nh), sizeof(gi_line_compact) * need));
    if (count) memcpy(nh, c->h_compact, sizeof(gi_line_compact) * count);
    if (c->h_compact) cudaFreeHost(c->h_compact);
    c->h_compact = nh;
    c->h_compact_cap = need;
  }
  if (host && !compact && c->h_lines_cap < (size_t)need) {
    gi_line* nh = nullptr;
    GI_CUDA(c, cudaMallocHost(reinterpret_cast<void**>(&nh), sizeof(gi_line) * need));
    if (count) memcpy(nh, c->h_lines, sizeof(gi_line) * count);
    if (c->h_lines) cudaFreeHost(c->h_lines);
    c->h_lines = nh;
    c->h_lines_cap = need;
  }
  auto put = [&](int64_t slot, const gi_line& L) -> gi_status {
    GI_CUDA(c, cudaMemcpy(d + slot, &L, sizeof(gi_line), cudaMemcpyHostToDevice));
    if (compact)
      c->h_compact[slot] = gi_line_compact{L.level_i, L.level_f, L.nu, L.S, L.A, L.I};
    else if (host)
      c->h_lines[slot] = L;
    return GI_OK;
  };
  for (size_t k = 0; k < upd.size(); k++) {
    gi_status s = put(upd_slot[k], upd[k]);
    if (s != GI_OK) return s;
  }
  for (const gi_line& L : add) {
    gi_status s = put(count++, L);
    if (s != GI_OK) return s;
  }
  // removals: the last line moves into each freed slot (highest slots first)
  std::sort(drop.begin(), drop.end(), std::greater<int64_t>());
  for (int64_t slot : drop) {
    const int64_t last = --count;
    if (slot != last) {
      gi_line L;
      if (host && !compact) {
        L = c->h_lines[last];
      } else {
        GI_CUDA(c, cudaMemcpy(&L, d + last, sizeof(gi_line), cudaMemcpyDeviceToHost));
      }
      gi_status s = put(slot, L);
      if (s != GI_OK) return s;
    }
  }
  c->nlines = count;
  *refined = (int64_t)n;
  return GI_OK;
}

}  // namespace gi
