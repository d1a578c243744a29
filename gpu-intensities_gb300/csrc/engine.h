// Internal declarations of the GB300 line-intensity engine (host side).
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <utility>
#include <vector>

#include "../../include/gi.h"

namespace gi {

// ------------------------------------------------------------------ memory
template <class T>
struct DevArray {
  T* p = nullptr;
  size_t n = 0;
  DevArray() = default;
  DevArray(const DevArray&) = delete;
  DevArray& operator=(const DevArray&) = delete;
  DevArray(DevArray&& o) noexcept : p(o.p), n(o.n) { o.p = nullptr; o.n = 0; }
  DevArray& operator=(DevArray&& o) noexcept {
    if (this != &o) { reset(); p = o.p; n = o.n; o.p = nullptr; o.n = 0; }
    return *this;
  }
  ~DevArray() { reset(); }
  void reset() {
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
  }
  cudaError_t alloc(size_t count) {
    reset();
    if (count == 0) count = 1;
    cudaError_t e = cudaMalloc(reinterpret_cast<void**>(&p), count * sizeof(T));
    if (e == cudaSuccess) n = count; else p = nullptr;
    return e;
  }
  // A pageable cudaMemcpy may return before its DMA lands; the legacy-stream
  // sync orders the copy before work on any (also non-blocking) stream.
  cudaError_t upload(const T* h, size_t count) {
    cudaError_t e = alloc(count);
    if (e != cudaSuccess || count == 0) return e;
    e = cudaMemcpy(p, h, count * sizeof(T), cudaMemcpyHostToDevice);
    return e != cudaSuccess ? e : cudaStreamSynchronize(cudaStreamLegacy);
  }
  cudaError_t upload(const std::vector<T>& v) { return upload(v.data(), v.size()); }
  // Like upload, but keeps the allocation (and so the address) when it is
  // large enough: tables a captured CUDA graph reads stay where they were.
  cudaError_t assign(const std::vector<T>& v) {
    cudaError_t e = reserve(std::max<size_t>(v.size(), 1));
    if (e != cudaSuccess || v.empty()) return e;
    e = cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice);
    return e != cudaSuccess ? e : cudaStreamSynchronize(cudaStreamLegacy);
  }
  // grow-only workspace
  cudaError_t reserve(size_t count) { return count <= n ? cudaSuccess : alloc(count); }
};

inline int round_up(int x, int m) { return (x + m - 1) / m * m; }

// ------------------------------------------------------------------ inputs
// One rotational/vibrational coupling term of the half line strength:
//   h[rF] += coef * Z_c[slotI][v(rF)]   (per final (k, tau) "key").
struct StencilTerm {
  int32_t slotI;
  int32_t c;
  double coef;
};

// One H build of a batched launch (launch_build_h's arguments); blk0 is its
// first block in the launch's 1-D grid, nblk its blocks (ldh/256 per kHCols
// of its ncol initial columns).
constexpr int kHCols = 16;  // initial columns per block of the batched H build
struct HItem {
  const double* Z;
  size_t zc;
  int ldz, nslotI, ndegF, nsizeF, ldh, Ntot, st_max, ncol;
  const int32_t *s_case, *case_ptr, *case_roots, *root_v, *root_key, *root_lam;
  const double* rep;
  const StencilTerm* st;
  const int32_t* st_n;
  double* H;
  long long blk0, nblk;
};
// One unit's Y rows of a batched digit build (split_build_y_digits' arguments):
// rows [row0, row0 + rows) of the round's Y.
struct YItem {
  const double* vecs;
  const int32_t* ivec;
  const int32_t *yptr, *yroot, *root_case, *root_lam, *case_iterm, *case_nelem;
  const double* rep;
  int ld, ndeg, Ntot, nslot;
  long long row0, rows;
};
// The column norms of several H in one launch: item k's columns are
// [col0, col0 + ncol) of the grid.
struct NormItem {
  const double* H;
  double* out;
  int ldh, n;
  long long col0, ncol;
};

// A line handed to the exact re-evaluation: initial vector i of the part's
// unit, final record f, and its slot in the line list (-1: not kept).
struct RefineRec {
  int32_t part, i, f, slot;
};

struct EpiParams {
  int jI, jF, ndegI, ndegF, reduced, combo_mask;
  double gns, zpe, beta, q_stat, fw0, fw1, thresh_S, thresh_I;
  double A_coef, intens_cm_mol, avogno;
  // exact re-evaluation of doubtful lines (refine.cu): the estimated error of
  // a transition moment per unit of its H column's norm, the relative
  // accuracy S must reach without it, the part (initial unit x final block)
  // the launch serves, and whether lines past that accuracy are handed over
  double err_coef, target;
  int part, refine_cond;
};

// One part of a final block's T in the fused epilogue of the persistent final
// GEMM: columns [c0, c1) hold the moments of nI initial levels of one unit,
// grp = ndegI * ndegF consecutive columns per level.
struct EpiPart {
  int c0, c1, grp, pad;
  const double* EI;     // the unit's initial energies
  const double* BI;     // their Boltzmann factors exp(-(E - zpe) beta)
  const int32_t* lvI;   // their line ids
  const double* hn;     // norms of the part's H columns
  EpiParams ep;
};

// Process-wide serial numbers: a captured launch sequence is tied to the
// exact basis objects it read.
uint64_t next_uid();

struct Basis {
  uint64_t uid = next_uid();
  int J = 0, D = 0, ncase = 0, max_deg = 0, mat_size = 0;
  std::vector<int32_t> icontr2icase, iroot, k, ktau, Nsym, Ntotal, ijterms;
  std::vector<std::vector<double>> repres;  // per gamma
  // derived
  std::vector<int32_t> root_key;    // 2k + tau (tau = ktau & 1)
  std::vector<int32_t> slot_of_key; // [2J+2] -> slot or -1
  int nslot = 0;
  std::vector<int32_t> case_ptr, case_roots;  // CSR: roots of each case
  std::vector<std::vector<int32_t>> s_case;   // per gamma: case of symmetrised s
  // device copies
  DevArray<int32_t> d_root_v, d_root_key, d_root_lam, d_root_case, d_case_ptr, d_case_roots;
  std::vector<DevArray<int32_t>> d_s_case, d_case_iterm, d_case_nelem;
  std::vector<DevArray<double>> d_rep;
  // (slot, v) -> roots CSR; depends on the dipole size N
  int y_N = -1;
  DevArray<int32_t> d_yptr, d_yroot;
  // largest iroot_correlat_j0 (checked against N without a pass over the roots)
  int32_t iroot_max = -1;
  // device copies of the key -> slot map and of the half-line-strength terms
  // towards J-1, J, J+1 ([jF - J + 1]; (2 jF + 2) * 6 terms and 2 jF + 2
  // counts), built when the basis or the 3j table is set
  DevArray<int32_t> d_slot_of_key;
  DevArray<StencilTerm> d_pair_st[3];
  DevArray<int32_t> d_pair_stn[3];
};

struct Block {
  int J = 0, gamma = 0, nsize = 0, nvec = 0, ld = 0;  // ld: padded row stride
  DevArray<double> d_vecs;                              // [nvec][ld], zero padded
  std::vector<double> energies;
  std::vector<int32_t> quanta;                          // [nvec][nmodes+1]
  DevArray<double> d_energies;
  // bf16 digit planes of the vectors for the split-precision path (cut on
  // first use, dropped when the block is replaced); digits_ev marks their
  // completion on the stream that cut them
  DevArray<uint16_t> d_digits;
  DevArray<int32_t> d_digit_exp;
  int digits_s = 0, digits_w = 0, digits_layout = -1;
  cudaEvent_t digits_ev = nullptr;
  // residency under a serving budget: an evicted block keeps its vectors in
  // pinned host memory and has no device arrays
  bool resident = true;
  double* h_vecs = nullptr;  // pinned [nvec][nsize]: the vectors while evicted, and
                             // kept after a restore, so that a later eviction of
                             // the same version copies nothing
  uint64_t h_version = ~0ull;  // the version h_vecs holds
  int pins = 0;              // running jobs that use the block
  uint64_t uid = next_uid(); // identity and vector version (serving Z cache)
  uint64_t version = 0;      // bumped whenever the vectors change
  uint64_t last_use = 0;     // serving clock of the last admission
  size_t device_bytes() const {
    return d_vecs.n * sizeof(double) + d_energies.n * sizeof(double) +
           d_digits.n * sizeof(uint16_t) + d_digit_exp.n * sizeof(int32_t);
  }
  ~Block() {
    if (digits_ev) cudaEventDestroy(digits_ev);
    if (h_vecs) cudaFreeHost(h_vecs);
  }
};

struct Level {
  int J, gamma, rec, ndeg, krot, taurot;
  double energy;
};

struct SplitState;  // split-precision state (split.cu)
struct Server;      // serving loop (serve.cu)
struct TroveMeta;   // level descriptors of a TROVE job (trove.cu)
struct DipoleStream;  // dipole kept in host memory, streamed in panels (stream.cu)

// One pair job of the serving loop: the lines of block (jI, gI) -> (jF, gF)
// under the filters of the whole loaded job (its ZPE and J range).
struct JobSel {
  bool on = false;
  int jI = 0, gI = 0, jF = 0, gF = 0;
  double zpe = 0.0;
  int jmin = 0, jmax = 0;
  double qstat = 0.0;  // partition function of the whole job (when QSTAT <= 0)
};

struct Ctx {
  SplitState* split = nullptr;
  int tune_mode = 0;          // split GEMM autotuner (gi_set_tuning)
  std::string tune_path;
  Ctx* parent = nullptr;      // a serving worker shares its parent's model state
  Server* server = nullptr;
  TroveMeta* trove = nullptr;
  std::mutex model_mu;        // guards lazily derived shared state (digits)
  std::mutex& mmu() { return parent ? parent->model_mu : model_mu; }
  JobSel job;
  int device = 0;
  size_t budget = 0;
  int nsm = 0;
  cudaStream_t stream = nullptr;      // where all device work is ordered
  cudaStream_t own_stream = nullptr;  // the context's own stream
  cudaEvent_t ev0 = nullptr, ev1 = nullptr;
  std::string err;

  int sym_type = 0, nrep = 0;
  std::vector<int32_t> degen;
  bool have_params = false;
  gi_params params{};

  int N = 0, Kp = 0;          // dipole size and padded row stride
  DevArray<double> d_mu;      // [3][N rows f][Kp]: row f holds mu_c(:, f)
  const double* mu() const { return parent ? parent->d_mu.p : d_mu.p; }
  DipoleStream* dstream = nullptr;  // set: the dipole stays in host memory
  bool streamed() const { return (parent ? parent->dstream : dstream) != nullptr; }

  std::map<int, std::shared_ptr<Basis>> bases;
  std::map<std::pair<int, int>, std::shared_ptr<Block>> blocks;

  int threej_jmax = -1;
  bool threej_user = false;
  std::vector<double> threej;

  // results of the last run
  std::vector<Level> levels;
  gi_line* h_lines = nullptr;  // pinned staging of the last run's lines
  size_t h_lines_cap = 0;
  DevArray<gi_line> d_lines;
  bool lines_on_device = false;
  // GI_RUN_COMPACT_LINES: the read-back is packed into d_compact on the
  // device, and the host receives 40-byte records in h_compact
  bool compact_lines = false;
  DevArray<gi_line_compact> d_compact;
  gi_line_compact* h_compact = nullptr;
  size_t h_compact_cap = 0;
  int64_t nlines = 0;
  gi_stats stats{};

  // per-phase device timing (GI_RUN_PHASE_TIMING)
  struct PhaseRec {
    int phase;
    cudaEvent_t a, b;
  };
  bool timing = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;
  std::vector<PhaseRec> phase_recs;
  cudaEvent_t take_event() {
    if (ev_used == ev_pool.size()) {
      cudaEvent_t e = nullptr;
      if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
      ev_pool.push_back(e);
    }
    return ev_pool[ev_used++];
  }

  // Line read-back overlapped with the run: after each final block's
  // epilogues the line count goes to ck_count[k] and ck_ev[k] is recorded; the
  // host copies every finished stretch of lines on d2h while later blocks run
  std::vector<cudaEvent_t> ck_ev;
  unsigned long long* ck_count = nullptr;  // pinned
  size_t ck_cap = 0;
  cudaStream_t d2h = nullptr;

  // CUDA graphs of captured launch sequences (GI_RUN_GRAPH), one per plan
  // signature, the most recently used first (at most kGraphCache): runs that
  // alternate between plans (the shards of a job) replay each one's graph
  struct GraphEntry {
    uint64_t sig = 0;
    cudaGraphExec_t exec = nullptr;
    gi_stats stats{};  // what the captured sequence adds to a run's counts
  };
  static constexpr size_t kGraphCache = 16;
  std::vector<GraphEntry> graphs;
  uint64_t gpending = 0;
  int64_t graph_replays = 0;
  // the part of the initial levels this run takes (gi_run_shard): levels at
  // positions l of the energy-sorted table with l % nshards == shard
  int shard = 0, nshards = 1;

  // workspaces
  DevArray<double> hls_v, hls_y, hls_z, hls_h;  // gi_half_ls (grow-only)
  double* hls_pin = nullptr;                     // its pinned host staging
  size_t hls_pin_cap = 0;
  // gi_half_ls: the launch sequence of a call shape, captured on its second
  // call and replayed while the shape and every buffer it names are unchanged
  struct HlsGraph {
    uint64_t sig;
    cudaGraphExec_t exec;
  };
  std::vector<HlsGraph> hls_graphs;  // most recently used first
  uint64_t hls_last_sig = 0;         // the last call run eagerly
  DevArray<int32_t> hls_iv;
  DevArray<double> w_y, w_z, w_h, w_t, w_EI;
  DevArray<unsigned long long> w_counter;
  DevArray<int32_t> w_ivec, w_int;
  DevArray<uint8_t> w_upper;
  DevArray<StencilTerm> w_stencil;
  DevArray<double> w_hn;       // H column norms of a group of final blocks
  DevArray<double> w_BI;       // Boltzmann factors of the run's initial levels
  DevArray<EpiPart> w_epi;     // parts of the fused epilogue
  DevArray<HItem> w_hitems;    // the H builds of every group (one launch per group)
  DevArray<long long> w_hfirst; // their first grid blocks, contiguous for the lookup
  DevArray<NormItem> w_nitems; // the H column norms of every group
  DevArray<YItem> w_yitems;    // the Y digit builds of every round (one launch per round)
  DevArray<RefineRec> w_rec;   // lines handed to the exact re-evaluation
  int64_t refine_max = 0;      // doubtful lines re-evaluated per run (gi_set_refine)
  DevArray<int32_t> w_stencil_n, w_levelI, w_levelF;
};

// Runs one launch group on the context's stream, counting it under `phase`
// and, when timing is on, bracketing it with CUDA events.
template <class F>
cudaError_t timed(Ctx* c, int phase, F&& launch) {
  c->stats.launches_phase[phase]++;
  c->stats.kernel_launches++;
  if (!c->timing) return launch();
  cudaEvent_t a = c->take_event(), b = c->take_event();
  if (!a || !b) return cudaErrorMemoryAllocation;
  cudaEventRecord(a, c->stream);
  cudaError_t e = launch();
  cudaEventRecord(b, c->stream);
  c->phase_recs.push_back({phase, a, b});
  return e;
}

// ------------------------------------------------------------------ host
gi_status fail(Ctx* c, gi_status s, const char* fmt, ...);
#define GI_CUDA(c, call)                                                                   \
  do {                                                                                     \
    cudaError_t e_ = (call);                                                               \
    if (e_ != cudaSuccess)                                                                 \
      return ::gi::fail((c), e_ == cudaErrorMemoryAllocation ? GI_ERR_NOMEM : GI_ERR_CUDA, \
                        "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), __FILE__, __LINE__); \
  } while (0)

// Sum of g_ns (2J+1) ndeg exp(-c2 (E - zpe) / T) over the loaded levels.
double partition_sum(const Ctx* c, double temperature, double zpe);
// Runs every block pair of the loaded job (or the one pair of c->job).
gi_status run_job(Ctx* c, int flags, int64_t* nlines_out);
// Builds the (slot, v) -> roots table of a basis for the context's dipole size.
gi_status ensure_ycsr(Ctx* c, Basis& b);
// Device tables of every basis's half-line-strength terms towards J-1, J, J+1
// (Basis::d_pair_st), from the context's 3j table where it covers the pair.
gi_status refresh_pair_tables(Ctx* c, Basis* only = nullptr);
// Serving: frees device memory for `bytes` more by evicting unpinned blocks
// other than `keep` and unused cached half line strengths (least recently
// used first).  Caller holds model_mu.
gi_status server_make_room(Ctx* c, size_t bytes, Block* keep);
// Serving Z cache: the half line strength Z = mu^T Y ([3][ncol][Kp], the run's
// layout) of an initial block for one selection of its vectors.  acquire
// (worker context, model lock not held) returns z = null when nothing can be
// cached; hit: z holds it, else the run writes it there.  release unpins it,
// keeping it valid after a successful run or dropping it otherwise.
struct ZEntry;
struct ZRef {
  ZEntry* e = nullptr;
  double* z = nullptr;
  bool hit = false;
};
gi_status zcache_acquire(Ctx* w, const Block* blk, const int32_t* ivec, int nI, size_t elems,
                         ZRef* out);
void zcache_release(Ctx* w, ZRef& r, bool ok);
// Stops the serving loop of c (if any): fails queued jobs, joins the workers.
gi_status server_stop(Ctx* c);
void trove_meta_release(Ctx* c);
// Frees a context's streams, events, pinned buffers and split state, then
// the context itself (its device arrays go with it).
void ctx_release(Ctx* c);

// The dipole in panels of rows f: fn(panel, component stride, rows, f0) is
// called in order, with stream `st` ordered after the panel's [3][rows][Kp]
// doubles are on the device.  A resident dipole is one panel of N rows.
using PanelFn = std::function<gi_status(const double*, size_t, int, int)>;
gi_status for_each_dipole_panel(Ctx* c, cudaStream_t st, const PanelFn& fn);
// Z_c = mu_c^T Y in FP64 (rows f of Z at ldz, components zc apart).
gi_status dipole_gemm_fp64(Ctx* c, const double* Y, int ldy, double* Z, int ldz, size_t zc,
                           int ncol, cudaStream_t st);
// Makes `pinned` (cudaMallocHost, [3][N][N] record order) the context's
// streamed dipole; the context frees it.
gi_status dipole_stream_adopt(Ctx* c, int N, double* pinned, int panel_rows);
void dipole_stream_release(Ctx* c);
int dipole_panel_rows(const Ctx* c);

// ------------------------------------------------------------------ kernels



cudaError_t launch_build_y(const double* vecs, int ld, const int32_t* ivec, int nI, int ndeg,
                           const Basis& b, int gamma, int degen, int N, int Kp, double* Y,
                           cudaStream_t s, int d0 = 0);
cudaError_t launch_build_h(const double* Z, size_t zstride_c, int ldz, int nslotI, int ndegI,
                           int nI, const Basis& bF, int gammaF, int degF, int nsizeF, int ldh,
                           const StencilTerm* st, const int32_t* st_n, int st_max, double* H,
                           cudaStream_t s);
HItem make_h_item(const double* Z, size_t zstride_c, int ldz, int nslotI, int ndegI, int nI,
                  const Basis& bF, int gammaF, int degF, int nsizeF, int ldh,
                  const StencilTerm* st, const int32_t* st_n, int st_max, double* H,
                  long long blk0);
// Every item of a device table in one launch (nblocks = the items' blocks).
cudaError_t launch_build_h_items(const HItem* items, const long long* firsts, int nitems,
                                 long long nblocks, cudaStream_t st);
cudaError_t launch_half_ls_prim(const double* Z, size_t zstride_c, int ldz, const Basis& bF,
                                const StencilTerm* st, const int32_t* st_n, int st_max,
                                double* h, cudaStream_t s);
// h from a Z held as K-split partial products Zp[p][col][c * cstride + v]
// (Zp already offset to the first column of the wanted degenerate component).
cudaError_t launch_half_ls_prim_parts(const double* Zp, int nparts, size_t pstride, int ldz,
                                      int cstride, const Basis& bF, const StencilTerm* st,
                                      const int32_t* st_n, int st_max, double* h,
                                      cudaStream_t s);

// out[k] = exp(-(E[k] - zpe) beta) (the epilogue's initial-level factor).
cudaError_t launch_pack_lines(const gi_line* in, gi_line_compact* out, long long n,
                              cudaStream_t st);
cudaError_t launch_boltz(const double* E, int n, double zpe, double beta, double* out,
                         cudaStream_t s);

// What the exact re-evaluation (refine.cu) needs of one epilogue part, an
// initial unit against one final block; host arrays live for the run.
struct RefinePart {
  const Block* bI;
  const Block* bF;
  const Basis* basI;
  const Basis* basF;
  int gI, gF;
  const int32_t* rec_i;  // the unit's initial record ids
  const int32_t* lvl_i;  // their line ids (level table index or record)
  const double* EI;      // their energies
  const int32_t* lvl_f;  // line id of every final record
  const StencilTerm* st_dev;
  const int32_t* stn_dev;
  EpiParams ep;
};
// Re-evaluates the n handed-over lines exactly and patches the run's line
// list (c->nlines, the device lines and, when the run copied them there, the
// host lines).
gi_status refine_lines(Ctx* c, const std::vector<RefinePart>& parts, const RefineRec* recs,
                       size_t n, int64_t* refined);
// counter[0]: lines kept, [1]: lines passing the filters, [2]: lines handed
// to the exact re-evaluation (records past rec_cap are counted, not stored).
// hn: the norms of the part's H columns (column (i ndegI + dI) ndegF + dF).
cudaError_t launch_epilogue(const double* T, int ldt, int nI, int nF, const int32_t* levelI,
                            const double* EI, const int32_t* levelF, const double* EF,
                            const uint8_t* upper_ok, const double* hn, const EpiParams& p,
                            gi_line* out, unsigned long long* counter, long long cap,
                            RefineRec* rec, long long rec_cap, cudaStream_t s);
// out[col] = || H[col * ldh + 0 .. n) ||_2 for col < ncol.
cudaError_t launch_col_norms(const double* H, int ldh, int n, int ncol, double* out,
                             cudaStream_t s);
// The same for the H of several final blocks in one launch (NormItem).
cudaError_t launch_col_norms_items(const NormItem* items, int nitems, long long ncol,
                                   cudaStream_t s);
// C[z][n*ldc + m] = sum_k A[z][m*lda + k] * B[n*ldb + k]; K multiple of 16.
cudaError_t gemm_fp64_nt(const double* A, int lda, size_t strideA, const double* B, int ldb,
                         double* C, int ldc, size_t strideC, int M, int Nc, int K, int batch,
                         cudaStream_t s);

// ------------------------------------------------------------------ host math
double three_j(int j1, int j2, int j3, int k1, int k2, int k3);
void precompute_threej(int jmax, std::vector<double>& out);
// Half-line-strength terms for every final key (2*jF+2 keys, 6 slots each);
// threej may be null, in which case three_j() supplies the values.
void stencil_fill(const Basis& bI, int jF, const double* threej, int tj_jmax, StencilTerm* st,
                  int32_t* st_n);

}  // namespace gi
