// Split-precision (Ozaki-style bf16 slice) GEMMs on the tcgen05 tensor pipe.
#pragma once
#include "engine.h"

namespace gi {
// Z[c][n*ldz + f] = sum_v mu_c(v, f) * Y[n*ldy + v] for c = 0..2, n < ncol.
// y_digits_ready: split_build_y_digits already wrote Y's digits (Y unused).
gi_status split_gemm_dipole(Ctx* c, const double* Y, int ldy, double* Z, int ldz, size_t zstride,
                            int ncol, bool y_digits_ready = false);
// The same for a few columns (the half line strength of single vectors), at
// the speed of one pass over the dipole digits: K is split into up to
// max_parts parts whose partial products go to Zp + part * part_stride, laid
// out [col][*ldz] with component c at rows c * (*ldz / 3); *nparts receives
// the number of parts to sum.
gi_status split_gemm_dipole_narrow(Ctx* c, const double* Y, int ldy, int ncol, double* Zp,
                                   size_t part_stride, int max_parts, int* nparts, int* ldz);
// Y of one unit (nI vectors of block `vecs`, ndeg components) built directly
// into rows [row0, row0 + nI * ndeg * nslot) of the Y digit set of a round of
// rows_total rows; split_fused_y() says when this path applies.
bool split_fused_y(const Ctx* c);
// Every unit's Y rows of a round (a device table of n items, rows in all) in
// one launch; rows_total as in split_build_y_digits.
gi_status split_build_y_digits_items(Ctx* c, const YItem* items, int n, long long rows,
                                     size_t rows_total);
gi_status split_build_y_digits(Ctx* c, const double* vecs, int ld, const int32_t* ivec, int nI,
                               int ndeg, const Basis& b, int gamma, size_t row0,
                               size_t rows_total);
// T[n*ldt + f] = sum_s V_F[f][s] * H[n*ldh + s] for the vectors of block fb
// (f < nvec, n < ncol); the block's digit planes are cut on first use.
gi_status split_gemm_final(Ctx* c, Block& fb, const double* H, int ldh, int ncol, double* T,
                           int ldt);
// The final-state GEMMs of several final blocks in one persistent launch:
// job j computes T_j[n*ldt_j + f] = sum_s V_Fj[f][s] * H_j[n*ldh_j + s].  The
// H digits of all jobs go to one workspace (split_reserve sizes it), so the
// jobs together may hold at most that many elements and columns, and at most
// split_grouped_max_jobs() of them.
struct FinalJob {
  Block* fb;
  const double* H;
  int ldh, ncol;
  double* T;
  int ldt;
  // the fused epilogue (split_gemm_final_grouped with lines != null): the
  // block's parts and its final levels' energies, upper flags and line ids
  const EpiPart* parts = nullptr;
  int nparts = 0;
  const double* EF = nullptr;
  const uint8_t* upper = nullptr;
  const int32_t* lvF = nullptr;
};
// Where the fused epilogue puts its lines (the stand-alone epilogue's
// arguments, epilogue.cuh).
struct FusedLines {
  gi_line* out;
  unsigned long long* counter;
  long long cap;
  RefineRec* rec;
  long long rec_cap;
};
bool split_grouped_final(const Ctx* c);  // the persistent grouped launch applies
int split_grouped_max_jobs();
int split_grouped_items(int nvec, int ncol);  // work items of one job
// With lines != null the epilogue warps form every job's lines (S, A, I,
// filters, thresholds) on the last K segment instead of storing T.
gi_status split_gemm_final_grouped(Ctx* c, const std::vector<FinalJob>& jobs,
                                   const FusedLines* lines = nullptr);
// The fused epilogue applies (GI_SPLIT_FUSED_EPI=0 turns it off).
bool split_fused_epilogue(const Ctx* c);
// Called once per run before the launch loop (sizes workspaces, slices the dipole).
gi_status split_prepare(Ctx* c);
// Before a launch sequence that must not allocate (graph capture): the B
// operand workspace for GEMMs of up to max_elems = ncol x K elements and
// max_cols columns, the digit planes of every final block in `finals`, and
// the kernels' shared-memory attributes.
gi_status split_reserve(Ctx* c, size_t max_elems, size_t max_cols,
                        const std::vector<Block*>& finals);
// Identity of the split state a captured launch sequence depends on (its
// workspaces, the dipole digits and the digit shape).
uint64_t split_identity(Ctx* c);
// Digit planes per operand the next split-precision run will use.
int split_digits(const Ctx* c);
void split_invalidate(Ctx* c);  // the dipole changed: drop its cached slices
// After a run: reads the device error word the split kernels set on a timeout.
gi_status split_check(Ctx* c);
// The device error word of the context's split GEMMs (nullptr before the
// first split-precision GEMM), for a read ordered on a stream.
const int* split_error_word(const Ctx* c);
void split_release(Ctx* c);
}  // namespace gi
