// The per-line epilogue shared by the stand-alone epilogue kernel (kernels.cu)
// and the epilogue warps of the persistent final-state GEMM (split.cu), so
// that both give the same bits: degeneracy sum, S, A_if, I(T), frequency
// window and thresholds (cuda_host.cu:1376-1408), the doubtful-line estimate,
// and a warp-aggregated append of kept lines and of lines handed to the exact
// re-evaluation.
#pragma once

#include <cuda_runtime.h>

#include "engine.h"

namespace gi {

struct LineEval {
  bool pass = false, keep = false, doubt = false, doubtful = false;
  gi_line L;
};

// t[dI + 2 dF] for the combinations in p.combo_mask, hnq[...] the norms of
// their H columns; ei, ef the level energies, boltz_i = exp(-(ei - zpe) beta);
// ok_f: the final level passes the upper filter.
__device__ __forceinline__ void eval_line(const EpiParams& p, const double* t, const double* hnq,
                                          double ei, double ef, double boltz_i, bool ok_f,
                                          int level_i, int level_f, LineEval& r) {
  r.pass = r.keep = r.doubt = r.doubtful = false;
  if (!ok_f) return;
  const double nu = ef - ei;
  if (!(nu >= p.fw0 && nu <= p.fw1)) return;
  r.pass = true;
  double ls = 0.0;
  for (int dF = 0; dF < p.ndegF; ++dF)
    for (int dI = 0; dI < p.ndegI; ++dI) ls += t[dI + 2 * dF] * t[dI + 2 * dF];
  ls /= (double)p.ndegI;
  if (p.reduced && p.ndegF != 1 && p.ndegI != 1) ls *= (double)p.ndegI;
  const double anu = fabs(nu);
  const double boltz_fc = anu * boltz_i * (1.0 - exp(-anu * p.beta)) / p.q_stat;
  const double A = p.A_coef * (double)(2 * p.jI + 1) * ls * (anu * anu * anu);
  const double S = ls * p.gns * (double)((2 * p.jI + 1) * (2 * p.jF + 1));
  const double In = S * p.intens_cm_mol * boltz_fc;
  r.keep = (S >= p.thresh_S) && (In / p.avogno >= p.thresh_I);
  // doubtful lines: the relative error of S estimated from the moments and
  // their columns' norms (an error of err_coef * |H col| per moment); a kept
  // line whose estimate passes the target, and any line whose S or I sits
  // within the estimate of a threshold, is re-evaluated exactly
  double num = 0.0, den = 0.0;
  for (int dF = 0; dF < p.ndegF; ++dF)
    for (int dI = 0; dI < p.ndegI; ++dI)
      if (p.combo_mask & (1 << (dI + 2 * dF))) {
        const double tq = t[dI + 2 * dF];
        num += fabs(tq) * hnq[dI + 2 * dF];
        den += tq * tq;
      }
  const double rel = den > 0.0 ? 2.0 * p.err_coef * num / den : 0.0;
  const double band = 4.0 * rel + 1e-14;
  const bool near_S = p.thresh_S > 0.0 && fabs(S - p.thresh_S) <= band * p.thresh_S;
  const double Im = In / p.avogno;
  const bool near_I = p.thresh_I > 0.0 && fabs(Im - p.thresh_I) <= band * p.thresh_I;
  r.doubtful = r.keep && rel > p.target;
  r.doubt = near_S || near_I || (r.doubtful && p.refine_cond);
  r.L.level_i = level_i;
  r.L.level_f = level_f;
  r.L.ndeg_i = p.ndegI;
  r.L.ndeg_f = p.ndegF;
  r.L.nu = nu;
  r.L.S = S;
  r.L.A = A;
  r.L.I = In;
#pragma unroll
  for (int q = 0; q < 4; ++q) r.L.t[q] = t[q];
}

// The warp's lines: counts, appends of kept lines, records of doubtful ones.
// Every lane of the warp calls it (r.pass false where a lane has no line).
// counter: [0] kept, [1] passing the filters, [2] handed over, [3] doubtful.
__device__ __forceinline__ void append_line(const LineEval& r, int part, int i, int f,
                                            gi_line* __restrict__ out,
                                            unsigned long long* counter, long long cap,
                                            RefineRec* __restrict__ rec, long long rec_cap) {
  const int lane = threadIdx.x & 31;
  const unsigned pmask = __ballot_sync(0xffffffffu, r.pass);
  if (pmask && lane == 0) atomicAdd(counter + 1, (unsigned long long)__popc(pmask));
  if (r.doubtful) atomicAdd(counter + 3, 1ull);
  const unsigned mask = __ballot_sync(0xffffffffu, r.keep);
  long long slot = -1;
  if (mask) {
    const int leader = __ffs(mask) - 1;
    unsigned long long base = 0;
    if (lane == leader) base = atomicAdd(counter, (unsigned long long)__popc(mask));
    base = __shfl_sync(0xffffffffu, base, leader);
    if (r.keep) {
      const unsigned long long pos = base + __popc(mask & ((1u << lane) - 1u));
      if ((long long)pos < cap) out[pos] = r.L;
      slot = (long long)pos;
    }
  }
  if (r.doubt) {
    const unsigned long long k = atomicAdd(counter + 2, 1ull);
    if ((long long)k < rec_cap) rec[k] = RefineRec{part, i, f, (int32_t)slot};
  }
}

}  // namespace gi
