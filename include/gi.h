/*
 * gi.h - C ABI of the GB300 line-intensity engine.
 *
 * One context drives one GPU.  The caller hands over the same inputs the
 * reference reads from TROVE checkpoints (vibrational dipole, per-J basis
 * tables, per-(J,Gamma) eigenvector blocks with energies and quanta) and the
 * parameters of its input deck; the engine returns the same lines (S, A_if,
 * I(T) and the transition moments) after the same filters.
 *
 * Conventions
 *   - Every call returns a gi_status; nothing exits the process.  The text of
 *     the last failure is available from gi_last_error().
 *   - All buffers are caller-owned; setters copy what they need (to device
 *     memory) before returning, so the caller may free its arrays afterwards
 *     (except a dipole passed with GI_DIPOLE_BORROW).
 *   - A context is used from one host thread at a time.
 *   - Indices are 0-based unless stated.  Symmetry indices gamma follow the
 *     reference's order for the group (e.g. C2V(M): A1, A2, B1, B2).
 *
 * Reference interfaces replaced (file:line in the reference project):
 *   gi_create/gi_destroy   dipole_initialise_gpu + device teardown
 *                          (cuda_host.cu:900-993, 1501-1503)
 *   gi_set_symmetry        read_symmetry (fields.cpp:11-115)
 *   gi_set_params          read_intensities / read_fields (fields.cpp:145-282)
 *   gi_set_dipole(_flipped) read_dipole_flipped + its upload
 *                          (trove_functions.cpp:113-205, cuda_host.cu:983)
 *   gi_set_dipole_streamed read_dipole_flipped_blocks + do_1st_half_ls_blocks
 *                          (trove_functions.cpp:207-310; cuda_host.cu:783-817)
 *   gi_set_basis           bset_contr_factory + correlate_index +
 *                          compute_ijterms + copy_bset_contr_to_gpu
 *                          (trove_functions.cpp:401-858, 927-966; cuda_host.cu:186-366)
 *   gi_set_threej          precompute_threej + copy_threej_to_gpu
 *                          (trove_functions.cpp:899-925; cuda_host.cu:379-383)
 *   gi_set_block           read_eigenvalues + the eigenvector fread/H2D
 *                          (trove_functions.cpp:1075-1429; cuda_host.cu:1196-1199, 1262-1273)
 *   gi_run                 dipole_do_intensities_async_omp
 *                          (cuda_host.cu:995-1506; declared cuda_host.cuh:19)
 *   gi_half_ls             do_1st_half_ls: device_correlate_vectors +
 *                          device_compute_1st_half_ls_flipped_dipole
 *                          (cuda_host.cu:767-780; dipole_kernals.cu:38-71, 162-227)
 *   gi_line / gi_level     the printed line and level record
 *                          (cuda_host.cu:1444-1473; trove_objects.h:113-127)
 */
#ifndef GI_H
#define GI_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum {
  GI_OK = 0,
  GI_ERR_ARG = 1,       /* invalid argument or inconsistent tables */
  GI_ERR_CUDA = 2,      /* CUDA runtime or kernel error */
  GI_ERR_NOMEM = 3,     /* device or pinned host allocation failed */
  GI_ERR_STATE = 4,     /* call out of order (e.g. run before inputs) */
  GI_ERR_BUDGET = 5,    /* the job does not fit the context's HBM budget */
  GI_ERR_NOTFOUND = 6,  /* unknown J / block / job id */
  GI_ERR_DEVICE = 7     /* a device-side check failed (status read back) */
} gi_status;

typedef enum { GI_PREC_FP64 = 0, GI_PREC_SPLIT = 1 } gi_precision;

typedef struct gi_ctx gi_ctx;

#define GI_MAX_REP 8
#define GI_MAX_MODES 16

/* The INTENSITY block of the reference's input deck (fields.h:176-210). */
typedef struct {
  double temperature;      /* K */
  double q_stat;           /* partition function */
  double ZPE;              /* cm^-1; < 0: the first J=0, Gamma=0 record energy */
  double erange_lower[2];  /* E-ZPE window of initial levels */
  double erange_upper[2];  /* E-ZPE window of final levels */
  double freq_window[2];   /* nu = E_F - E_I window */
  double gns[GI_MAX_REP];  /* nuclear-spin weights; <= 1e-8 disables the symmetry */
  int32_t isym_pairs[GI_MAX_REP]; /* SELECTION */
  int32_t nmodes;
  int32_t quanta_lower[2][GI_MAX_MODES]; /* [0]=min, [1]=max of quanta[1..nmodes] */
  int32_t quanta_upper[2][GI_MAX_MODES];
  int32_t reduced;         /* SYMMETRY REDUCED */
  int32_t precision;       /* gi_precision */
  int32_t split_slices;    /* bf16 slices per FP64 operand in GI_PREC_SPLIT (0: default) */
  int32_t reserved;
  double thresh_linestrength; /* keep lines with S >= this (Debye^2) */
  double thresh_intensity;    /* keep lines with I >= this (cm/molecule) */
} gi_params;

/* One output line (cuda_host.cu:1444-1473).  level_i/level_f index the
   energy-sorted level table (gi_get_levels). */
typedef struct {
  int32_t level_i, level_f;
  int32_t ndeg_i, ndeg_f;
  double nu;   /* E_F - E_I, cm^-1 */
  double S;    /* line strength, Debye^2 */
  double A;    /* Einstein A, 1/s */
  double I;    /* absorption intensity, cm/mol (as the reference prints) */
  double t[4]; /* transition moments, Debye: t[ideg_i + 2*ideg_f] */
} gi_line;

/* The compact form of a line (GI_RUN_COMPACT_LINES): the fields a line list
   needs, 40 bytes instead of 80 (no degeneracies, no transition moments). */
typedef struct {
  int32_t level_i, level_f;
  double nu, S, A, I;
} gi_line_compact;

/* One level (TO_PTeigen, trove_objects.h:113-127). */
typedef struct {
  int32_t J, gamma;
  int32_t rec;        /* 0-based record (vector) index within its block */
  int32_t ndeg;
  int32_t krot, taurot;
  double energy;      /* absolute, cm^-1 */
} gi_level;

/* Phases of a run, for per-phase device timing (GI_RUN_PHASE_TIMING). */
enum {
  GI_PHASE_CORRELATE = 0, /* symmetrised -> primitive + scatter (initial vectors) */
  GI_PHASE_HALFLS_GEMM,   /* Z = mu^T Y, the dense part of the half line strength */
  GI_PHASE_STENCIL,       /* 3j/K-tau combination + projection onto the final basis */
  GI_PHASE_FINAL_GEMM,    /* T = V_F^T H, the final-state contraction */
  GI_PHASE_EPILOGUE,      /* S, A, I, filters, line output */
  GI_PHASE_SLICE,         /* FP64 -> bf16 slice conversion (split precision) */
  GI_NPHASE
};

typedef struct {
  int64_t nlines;          /* lines returned (after the thresholds) */
  int64_t nlines_filtered; /* lines passing every filter, before the thresholds */
  int64_t npairs_checked;  /* (i, f) pairs that passed the block-level rules */
  int32_t nblock_pairs;
  int32_t nlevels;
  double zpe;
  double seconds_total;    /* wall time of the last gi_run */
  double seconds_gpu;      /* device time of the last gi_run (CUDA events) */
  double flops_halfls;     /* algorithmic FP64 flops of the half line strength */
  double flops_final;      /* algorithmic FP64 flops of the final contraction */
  double flops_tensor;     /* bf16 tensor flops of the split-precision GEMMs: digit-pair
                              products x 2 x the true (unpadded) M, N and K */
  double bytes_correlate;  /* algorithmic HBM bytes of the correlate phase */
  double seconds_phase[GI_NPHASE]; /* device time per phase (GI_RUN_PHASE_TIMING) */
  int32_t launches_phase[GI_NPHASE];
  int32_t kernel_launches; /* kernels launched by the last gi_run */
  int32_t reserved;
  int64_t nlines_doubtful; /* kept lines whose estimated relative error of S passes the
                              accuracy target (1e-12 FP64, 1e-11 split) */
  int64_t nlines_handed;   /* lines handed to the exact re-evaluation: lines within their
                              error of a threshold, and doubtful lines up to the refine limit */
  int64_t nlines_refined;  /* of those, re-evaluated (all unless the record buffer overflowed) */
} gi_stats;

/* Context ---------------------------------------------------------------- */
gi_status gi_create(gi_ctx** out, int device, size_t hbm_budget_bytes);
gi_status gi_destroy(gi_ctx* ctx);
/* Orders all later device work of the context (runs, half line strengths,
 * uploads' consumers) on the caller's cudaStream_t `stream`; NULL returns to
 * the context's own stream.  Waits for work already queued on the previous
 * stream.  The stream must belong to the context's device and outlive its use.
 * No counterpart in the reference, whose kernels run on its own streams
 * (cuda_host.cu:980-992). */
gi_status gi_set_stream(gi_ctx* ctx, void* stream);
/* Autotuner of the split-precision GEMM launch configuration (one- or
 * two-pass kernel, L2 raster group) per shape class (digits, row tiles,
 * power-of-two column bucket, K).  mode 0 (default): configurations from the
 * table, a fixed default for classes not in it; mode 1: the first GEMM of a
 * class not in the table times every candidate on its operands (CUDA events)
 * and keeps the fastest.  path (optional, may be NULL): a text file the table
 * is read from and written to.  The table is shared by all contexts of the
 * process.  Tuning is skipped inside a CUDA-graph capture.  No counterpart in
 * the reference (fixed launch shapes, dipole_kernals.cu:162-227). */
gi_status gi_set_tuning(gi_ctx* ctx, int mode, const char* path);
/* Exact re-evaluation of doubtful lines.  Every transition moment carries an
 * error of a few units of FP64 rounding of its H column's norm; a line whose
 * moment cancels far below that column (its estimated relative error of S
 * passes 1e-12 on the FP64 path or 1e-11 split) is doubtful.  With
 * max_lines > 0 up to that many doubtful lines per run are recomputed in
 * double-double arithmetic (their initial column's half line strength, the
 * final dot) and their S, A, I replaced; 0 (the default) leaves them at the
 * GEMM paths' accuracy.  Independently of this setting, every line whose S or
 * I lies within its estimated error of a threshold is re-evaluated before the
 * keep decision, so line selection does not depend on rounding.  Counts are in
 * gi_stats.  No counterpart in the reference, which evaluates every line in
 * plain FP64 (cuda_host.cu:1301-1317). */
gi_status gi_set_refine(gi_ctx* ctx, int64_t max_lines);
const char* gi_last_error(const gi_ctx* ctx);
const char* gi_status_string(gi_status s);

/* Inputs ------------------------------------------------------------------ */
/* sym_type: 1 C2V(M), 2 C3V(M), 3 D3H(M) as in the reference deck. */
gi_status gi_set_symmetry(gi_ctx* ctx, int sym_type);
gi_status gi_set_params(gi_ctx* ctx, const gi_params* p);
/* mu: [3][N*N] doubles in the checkpoint's record order, mu_c(i,f) at
   c*N*N + i + f*N (c = x, y, z). */
gi_status gi_set_dipole(gi_ctx* ctx, int N, const double* mu);
/* The same dipole in the reference's in-memory layout after
   read_dipole_flipped (trove_functions.cpp:113-205): dip[f + i*N + c*N*N] =
   mu_c(i, f), i.e. FintensityJob::dipole_me. */
gi_status gi_set_dipole_flipped(gi_ctx* ctx, int N, const double* dip);
/* A dipole that stays in host memory (N beyond what the device should hold):
   the split-dipole path of the reference (read_dipole_flipped_blocks,
   trove_functions.cpp:207-310; do_1st_half_ls_blocks, cuda_host.cu:783-817;
   chosen above max_dipole_size, cuda_host.cu:10,858-867).  mu is in
   gi_set_dipole's record order.  Every half-line-strength contraction streams
   it through the device in panels of `panel_rows` rows f (all three
   components), double-buffered on a copy stream so that the copy of panel
   p+1 overlaps the contraction of panel p; 0 picks rows for about
   GI_DIPOLE_PANEL_BYTES of device staging.  Results are bit-identical to the
   resident dipole's.  By default the engine keeps a pinned copy of mu; with
   GI_DIPOLE_BORROW it page-locks and reads the caller's array instead, which
   must then stay valid and unchanged until the dipole is replaced or the
   context destroyed.  Runs are issued eagerly (GI_RUN_GRAPH is ignored) and
   a streamed dipole cannot be served (gi_serve_start fails). */
#define GI_DIPOLE_BORROW 1
#define GI_DIPOLE_PANEL_BYTES ((size_t)4 << 30)
gi_status gi_set_dipole_streamed(gi_ctx* ctx, int N, const double* mu, int panel_rows, int flags);
/* Rows per panel of a streamed dipole (0: resident dipole). */
int gi_dipole_panel_rows(const gi_ctx* ctx);
/* The per-J contracted basis (TO_bset_contrT):
     icontr2icase[2*D]:   [r] = case, [r+D] = lambda (degenerate component)
     iroot_correlat_j0[D], k[D], ktau[D] (= 2k+tau)
     Nsym[nrep*ncase]:    N[g + case*nrep]
     Ntotal[nrep]
     repres[g]:           Ntotal[g]*degen[g]*mat_size doubles,
                          (s, ideg, lambda) at s + ideg*Ntot + lambda*degen*Ntot */
gi_status gi_set_basis(gi_ctx* ctx, int J, int D, int ncase, int max_deg_size, int mat_size,
                       const int32_t* icontr2icase, const int32_t* iroot_correlat_j0,
                       const int32_t* k, const int32_t* ktau, const int32_t* Nsym,
                       const int32_t* Ntotal, const double* const* repres);
/* Optional: a 3j table laid out as precompute_threej(jmax); by default the
   engine computes the same table itself. */
gi_status gi_set_threej(gi_ctx* ctx, int jmax, const double* threej);
/* One (J, gamma) block: vecs[nvec][nsize] (record irec = row irec-1),
   energies[nvec], quanta[nvec][nmodes+1] (quanta[0] = rotational index). */
gi_status gi_set_block(gi_ctx* ctx, int J, int gamma, int nsize, int nvec, const double* vecs,
                       const double* energies, const int32_t* quanta);

/* The same, with vecs_dev a device pointer of the context's GPU
   (vecs_dev[nvec][nsize], e.g. an eigensolver's output already in HBM); the
   engine copies it device to device.  No counterpart in the reference, which
   reads every vector from disk (cuda_host.cu:1196-1199). */
gi_status gi_set_block_device(gi_ctx* ctx, int J, int gamma, int nsize, int nvec,
                              const double* vecs_dev, const double* energies,
                              const int32_t* quanta);

/* Run ---------------------------------------------------------------------- */
#define GI_RUN_LINES_ON_DEVICE 1 /* keep lines in device memory (no D2H) */
#define GI_RUN_PHASE_TIMING 2    /* time every kernel with CUDA events (gi_stats) */
#define GI_RUN_GRAPH 4           /* launch the job's kernels as one CUDA graph: captured on
                                    the first run of a plan, replayed while the plan (blocks,
                                    parameters, sizes, buffers) is unchanged; ignored with
                                    GI_RUN_PHASE_TIMING */
#define GI_RUN_COMPACT_LINES 8   /* the lines read back to host memory during the run are
                                    gi_line_compact records (half the bytes); read them
                                    with gi_get_lines_compact */
/* Computes every line of the job (all loaded J; |dJ| <= 1; the reference's
   filters).  *nlines receives the count. */
gi_status gi_run(gi_ctx* ctx, int flags, int64_t* nlines);
/* The part of the job whose initial levels sit at positions l of the
   energy-sorted level table with l % nshards == shard: the reference's split
   of the initial levels over devices (dipole_do_intensities_async_omp(job,
   device_id, num_devices), cuda_host.cu:995, its loop at cuda_host.cu:1174).
   The union of the shards 0..nshards-1 is the job's lines; ZPE, the level
   table and the partition function are the whole job's.  A batch of work for
   one GPU (one shard per step) or one of several GPUs (one shard per rank).
   gi_run(ctx, flags, n) is gi_run_shard(ctx, flags, 0, 1, n). */
gi_status gi_run_shard(gi_ctx* ctx, int flags, int shard, int nshards, int64_t* nlines);
gi_status gi_get_lines(gi_ctx* ctx, int64_t offset, int64_t count, gi_line* out);
/* The last run's lines as compact records.  After a run with
   GI_RUN_COMPACT_LINES (and without GI_RUN_LINES_ON_DEVICE) they are already
   in host memory; otherwise they are converted from the full records.
   gi_get_lines still returns the full records after a compact run (copied
   from device memory, where the full records stay until the next run). */
gi_status gi_get_lines_compact(gi_ctx* ctx, int64_t offset, int64_t count, gi_line_compact* out);
/* Orders the last run's lines by (initial level, final level), the order of
   the reference's single-device loop (cuda_host.cu:1174-1473); the run
   itself appends lines in the order its blocks finish. */
gi_status gi_sort_lines(gi_ctx* ctx);
gi_status gi_num_levels(gi_ctx* ctx, int32_t* n);
gi_status gi_get_levels(gi_ctx* ctx, int32_t cap, gi_level* out);
gi_status gi_get_stats(gi_ctx* ctx, gi_stats* out);

/* Kernel-level drop-in for do_1st_half_ls: half line strength of one initial
   vector vsym (nsize doubles of block (jI, gammaI)), degenerate component
   ideg, towards the J=jF basis; half_ls receives D_F doubles. */
gi_status gi_half_ls(gi_ctx* ctx, int jI, int gammaI, int ideg, int jF, const double* vsym,
                     double* half_ls);

/* Allocation-free variant of gi_half_ls.  No counterpart in the reference.
   For callers that cannot allocate device memory when they compute a half
   line strength: a serving loop whose HBM is fully reserved by its admission
   budget, a host framework or eigensolver that owns device memory through its
   own pool, or a latency-sensitive caller that cannot afford the implicit
   device-wide synchronisation of cudaMalloc/cudaFree.  The call allocates
   nothing: vsym_dev (nsize doubles of block (jI, gammaI)) and half_ls_dev
   (D_F doubles) are device buffers the caller owns, and the scratch is one
   fixed device array of GI_NOALLOC_SCRATCH_BYTES inside the library, held by
   every GPU that loads it until the process exits.  Limit: degen(gammaI) *
   (number of (k, tau) slots of J=jI) * round_up(N, 64) <= 2^19; larger sizes
   return GI_ERR_ARG (use gi_half_ls).  The rotational term tables it reads
   are built by gi_set_basis / gi_set_threej, so the call copies nothing from
   the host: the work is enqueued on `stream` (a cudaStream_t; NULL = the
   context's stream) and the call returns without waiting.  All calls share
   the scratch array, which keeps the last call's contents: calls whose work
   overlaps on the GPU race, so order them (one stream, or events).  The first
   call on a device looks up the array's device address once
   (cudaGetSymbolAddress) with that device current; make that first call
   before any stream capture. */
#define GI_NOALLOC_SCRATCH_BYTES (16u << 20)
gi_status gi_half_ls_noalloc(gi_ctx* ctx, int jI, int gammaI, int ideg, int jF,
                             const double* vsym_dev, double* half_ls_dev, void* stream);

/* TROVE job files and the reference's text interfaces ----------------------- */
/* The input deck (read_fields / read_intensities, fields.cpp:11-282): NMODES,
 * SYMGROUP and the INTENSITY block (TEMPERATURE, QSTAT, ZPE, J, FREQ-WINDOW,
 * ENERGY LOW/UPPER, GNS, SELECTION, THRESH_LINE, V n LOWER/UPPER, SYMMETRY
 * REDUCED).  Fields the deck leaves out get open windows, g_ns = 1,
 * T = 296 K, QSTAT = 1 and no threshold (the reference leaves them
 * uninitialised).  Host only; err (optional) receives a message. */
typedef struct {
  int32_t sym_type;  /* 1 C2V(M), 2 C3V(M), 3 D3H(M) */
  int32_t nmodes;
  int32_t jvals[2];  /* the deck's "J j0 j1" */
  gi_params params;
} gi_deck;
gi_status gi_deck_parse(const char* text, gi_deck* deck, char* err, size_t err_cap);

#define GI_TROVE_MAXQ 17 /* quanta(0:nmodes) entries kept per level */
typedef struct {
  int32_t irec[2];     /* records of the degenerate components, 1-based */
  int32_t ilevel;      /* level index within its file, 0-based */
  int32_t ndeg;
  int32_t krot, taurot;
  int32_t large_coef;
  int32_t reserved;
  double energy;
  int32_t quanta[GI_TROVE_MAXQ];  /* quanta(0:nmodes); quanta(0) the rotational index */
  int32_t cgamma[GI_TROVE_MAXQ];  /* symmetry of each class (0:nclasses), 0-based */
  int32_t normal[GI_TROVE_MAXQ];  /* normal-mode quanta (0:nmodes) */
} gi_trove_level;

/* Host-only readers of TROVE checkpoints in `dir` (no GPU needed):
 *   gi_trove_read_basis   j0eigen_quanta<J>.chk with J=0's for the root
 *                         correlation (bset_contr_factory + correlate_index,
 *                         trove_functions.cpp:401-858).  dims receives
 *                         {D, ncase, max_deg_size, mat_size, nclasses, N}; the
 *                         arrays (any may be NULL) have gi_set_basis's layout.
 *   gi_trove_read_dipole  j0_extfield.chk (trove_functions.cpp:113-205), in
 *                         gi_set_dipole's record order.
 *   gi_trove_read_levels  j0eigen_descr<J>_<gamma+1>.chk (read_eigenvalues,
 *                         trove_functions.cpp:1075-1429): one entry per level
 *                         (ideg = 1 line) in file order; call with out = NULL
 *                         for the count. */
gi_status gi_trove_read_basis(const char* dir, int J, int sym_type, int32_t* dims, int32_t* k,
                              int32_t* ktau, int32_t* iroot_correlat_j0, int32_t* icontr2icase,
                              int32_t* Nsym, int32_t* Ntotal, double* const* repres, char* err,
                              size_t err_cap);
gi_status gi_trove_read_dipole(const char* dir, int N, double* mu, char* err, size_t err_cap);
gi_status gi_trove_read_levels(const char* dir, int J, int gamma, int sym_type, int nmodes,
                               int nclasses, int32_t* n, int32_t* dim_basis, gi_trove_level* out,
                               int32_t cap_levels, char* err, size_t err_cap);

#define GI_TROVE_ALL_J 1 /* load every J in [j0, j1], not only j0 and j1 */
/* keep the dipole in host memory and stream it (gi_set_dipole_streamed with
   the default panel); also chosen when the padded dipole would take more than
   half of the device's memory */
#define GI_TROVE_STREAM_DIPOLE 2
/* Loads a TROVE job into the context: symmetry and parameters from the deck
 * (keeping the context's precision choice), the J=0 basis, the bases of the
 * deck's J values, the dipole, and one block per (J, gamma) with g_ns > 0 holding
 * every level of its descr file (ideg = 1 record of each, from the vectors
 * file).  Replaces dipole_initialise_cpu + the per-level fread
 * (cuda_host.cu:837-898, 1196-1199). */
gi_status gi_load_trove(gi_ctx* ctx, const char* dir, const gi_deck* deck, int flags);
/* The lines [offset, offset+count) of the last gi_run (lines with level-table
   ids) as the reference prints them (cuda_host.cu:1444-1473), one per text
   line; *used receives the bytes needed (without the final NUL). */
gi_status gi_format_lines(gi_ctx* ctx, int64_t offset, int64_t count, char* buf, size_t cap,
                          size_t* used);
/* The fields of one printed line (cuda_host.cu:1444-1473) and the formatter
   gi_format_lines applies to them, host code only (no context, no GPU).  The
   branch letter follows from jF - jI; energies are relative to the ZPE;
   labels hold the symmetry names of classes 0..nclasses, quanta and normal
   indices 1..nmodes (index 0 unused, as in gi_trove_level); ilevel is
   0-based (printed + 1); t holds ndeg_i * ndeg_f moments t[dI + 2 dF]. */
typedef struct {
  int32_t jF, jI, krotF, krotI, ilevelF, ilevelI;
  int32_t nclasses, nmodes, ndegF, ndegI;
  const char* symF;
  const char* symI;
  const char* cgF[GI_TROVE_MAXQ];
  const char* cgI[GI_TROVE_MAXQ];
  int32_t quantaF[GI_TROVE_MAXQ], quantaI[GI_TROVE_MAXQ];
  int32_t normalF[GI_TROVE_MAXQ], normalI[GI_TROVE_MAXQ];
  double eF, eI, nu, S, A, I;
  double t[4];
} gi_line_text;
/* Appends the line's text ("\n"-terminated) to buf; *used receives its
   length (also when cap is too small, then GI_ERR_ARG). */
gi_status gi_format_line_text(const gi_line_text* f, char* buf, size_t cap, size_t* used);
/* Partition function over the loaded levels: sum of g_ns(gamma) (2J+1) ndeg
   exp(-c2 (E - ZPE) / T); the reference takes it from the deck (QSTAT).  A run
   whose q_stat is <= 0 uses this value at its temperature. */
gi_status gi_partition_function(gi_ctx* ctx, double temperature, double* q);

/* Serving ----------------------------------------------------------------- */
/* No counterpart in the reference, which processes one (J, J+1) job per
 * process (main.cu:34-95).  A serving context takes intensity jobs of single
 * block pairs (J, Gamma) -> (J', Gamma') as an upstream eigensolver finishes
 * blocks, and runs up to `slots` of them at once, each on its own stream, so
 * their work overlaps on the GPU.  Jobs are admitted in arrival order when a
 * slot is free and their blocks fit the budget; blocks stay resident in HBM
 * and the least recently used blocks that no running job holds move to pinned
 * host memory when room is needed.  A job's lines are the lines of that block
 * pair that gi_run over all loaded blocks produces (same filters, ZPE and J
 * range), with level_i / level_f holding record indices within the two blocks.
 * The half line strength of an initial block (its Z = mu^T Y, the GEMM most of
 * a job's work goes to) is kept in a cache under the same budget and shared by
 * later jobs that start from the same block with the same selection of its
 * vectors (until the block's vectors change); cached entries and blocks are
 * evicted together, least recently used first (GI_SERVE_NO_ZCACHE turns the
 * cache off).
 * While serving, gi_set_block / gi_set_block_device / gi_set_params (except
 * precision and split_slices) / gi_submit and the job calls may be used from
 * the context's thread; the other setters and gi_run return GI_ERR_STATE. */
#define GI_SERVE_NO_ZCACHE 1 /* do not keep initial blocks' half line strengths */
typedef struct {
  int32_t slots;                /* jobs in flight, one stream each (0: 3) */
  int32_t flags;                /* GI_SERVE_* */
  size_t hbm_budget_bytes;      /* device bytes for resident blocks and slot
                                   workspaces (0: the context's budget, else
                                   80 % of the free memory) */
  size_t slot_workspace_bytes;  /* workspace cap per slot (0: budget / (4 slots)) */
} gi_serve_config;

#define GI_JOB_QUEUED 0
#define GI_JOB_RUNNING 1
#define GI_JOB_DONE 2
#define GI_JOB_FAILED 3

typedef struct {
  int32_t state;              /* GI_JOB_* */
  int32_t status;             /* gi_status of a finished job */
  int64_t nlines;             /* lines kept (after the intensity threshold) */
  int64_t nlines_filtered;    /* lines that passed the selection filters */
  double seconds_queued;      /* submit -> admission */
  double seconds_latency;     /* submit -> done (or -> now while in flight) */
  double seconds_gpu;         /* device time of the job's launch sequence */
} gi_job_info;

typedef struct {
  int64_t submitted, completed, failed;
  int64_t lines, lines_filtered;
  int64_t evictions, restores;  /* blocks moved to / back from pinned host */
  int32_t queued, running;
  double latency_p50, latency_p99, latency_mean, latency_max;  /* seconds */
  double queue_p50, queue_p99;
  size_t resident_bytes, peak_resident_bytes, budget_bytes, slot_workspace_bytes;
  int32_t slots;
  int32_t reserved;
  /* the Z cache: jobs whose initial block's half line strength was cached
     (hits) or computed (misses), entries dropped for room, bytes held */
  int64_t zcache_hits, zcache_misses, zcache_evictions;
  size_t zcache_bytes;
} gi_serve_stats;

gi_status gi_serve_start(gi_ctx* ctx, const gi_serve_config* cfg);
/* Waits for the running jobs; queued jobs fail with GI_ERR_STATE. */
gi_status gi_serve_stop(gi_ctx* ctx);
gi_status gi_submit(gi_ctx* ctx, int jI, int gammaI, int jF, int gammaF, uint64_t* job_id);
/* Waits up to timeout_s seconds (< 0: without limit) for the job to finish;
   info (optional) receives its state.  Returns the job's status once done. */
gi_status gi_job_wait(gi_ctx* ctx, uint64_t job_id, double timeout_s, gi_job_info* info);
gi_status gi_job_lines(gi_ctx* ctx, uint64_t job_id, int64_t offset, int64_t count,
                       gi_line* out);
/* Forgets a finished job and its lines. */
gi_status gi_job_release(gi_ctx* ctx, uint64_t job_id);
/* Latency percentiles over the jobs finished since start / the last reset. */
gi_status gi_serve_get_stats(gi_ctx* ctx, gi_serve_stats* out);
gi_status gi_serve_reset_stats(gi_ctx* ctx);

#ifdef __cplusplus
}
#endif
#endif /* GI_H */
