/*
 * CPU oracle for the line-intensity hot path: a plain-C restatement of the
 * reference's algorithm, used ONLY as test infrastructure (tests/, the
 * smoke check and the CPU-baseline leg of bench.py).  The product never
 * links or calls this code.
 *
 * Parity pinning: the reference ships no tests, fixtures or golden vectors
 * for this path.  The 3j routine here is pinned bit-for-bit against the
 * reference's own three_j/precompute_threej compiled from its sources
 * (oracle/build_ref.sh -> oracle/_ref/); the rest follows the reference's
 * kernels and driver loop line by line (citations on each function).
 *
 * Accuracy: or_correlate / or_half_ls / or_dot (the kernel-level functions
 * pinned against the reference's kernels) use Ogita-Rump-Oishi Dot2 (TwoProd
 * via fma + TwoSum).  or_run with precise = 1 (the checker) carries the
 * correlated vectors and the half line strength as double-double values into
 * a double-double final dot, so a transition moment is accurate far below
 * FP64 rounding of its terms and tolerances measure the engine, also on lines
 * whose moment cancels.  With precise = 0 it is the reference's plain FP64
 * arithmetic (the CPU baseline port).
 */
#ifndef GI_ORACLE_H
#define GI_ORACLE_H
#include <stddef.h>
#include <stdint.h>
#ifdef __cplusplus
extern "C" {
#endif

/* Per-J contracted basis tables (trove_objects.h:88-111, cuda_objects.cuh:5-21). */
typedef struct {
  int jval;
  int Maxcontracts;        /* D_J: primitive roots */
  int Maxsymcoeffs;        /* number of "cases" (rows of icontr2icase) */
  int max_deg_size;
  int mat_size;            /* third extent of repres */
  const int32_t* icontr2icase;      /* [2*D]: [r] = icase, [r+D] = ilambda */
  const int32_t* iroot_correlat_j0; /* [D]: J=0 vibrational index of root r */
  const int32_t* k;                 /* [D] */
  const int32_t* ktau;              /* [D] = 2k+tau */
  const int32_t* Nsym;              /* [nrep*Maxsymcoeffs]: N[g + icase*nrep] */
  const int32_t* Ntotal;            /* [nrep] */
  const double* const* repres;      /* [nrep] -> [Ntotal*degen*mat_size],
                                       element (s, ideg, ib) at s + ideg*Ntot + ib*degen*Ntot */
} or_basis;

/* One (J, Gamma) eigenvector block: the vectors file and its descr records. */
typedef struct {
  int nsize;               /* symmetrised dimension */
  int nvec;                /* records (levels) */
  const double* vecs;      /* [nvec][nsize]; record irec (1-based) = row irec-1 */
  const double* energies;  /* [nvec] in record order */
  const int32_t* quanta;   /* [nvec][nmodes+1]; quanta[0] = rotational index */
} or_block;

/* The intensity job (fields.h:176-210), restricted to what the path reads. */
typedef struct {
  int sym_type;            /* 1 C2V(M), 2 C3V(M), 3 D3H(M) (fields.h:136-138) */
  int nrep;
  const int32_t* degen;    /* [nrep] */
  int nmodes;
  double ZPE;              /* < 0: taken from the J=0, Gamma=0 records */
  double erange_lower[2], erange_upper[2];
  double freq_window[2];
  int jvals[2];
  double q_stat, temperature;
  const double* gns;       /* [nrep]; gns <= 1e-8 switches the symmetry off */
  const int32_t* isym_pairs; /* [nrep] */
  int reduced;
  const int32_t* quanta_lower; /* [2*nmodes]: [0..nmodes) lower bounds, [nmodes..) upper */
  const int32_t* quanta_upper; /* [2*nmodes] */
  double thresh_linestrength;  /* keep S >= this (Debye^2) */
  double thresh_intensity;     /* keep I/N_A >= this (cm/molecule) */
  int N;                   /* J=0 basis size */
  const double* mu;        /* [3][N*N]: mu_c(i,f) at c*N*N + i + f*N (record order) */
  or_basis basis[2];       /* for jvals[0], jvals[1] */
  const or_block* blocks;  /* [2*nrep]: index jind + 2*gamma */
  int nthreads;            /* OpenMP threads (<=0: library default) */
  int precise;             /* 1: double-double reductions (the checker);
                              0: the reference's plain FP64 sums (the timed port) */
} or_job;

typedef struct {
  int32_t jI, gammaI, recI;   /* recI: 0-based record in the (jI, gammaI) block */
  int32_t jF, gammaF, recF;
  int32_t ndegI, ndegF;
  double nu;                  /* E_F - E_I */
  double S, A, I;             /* Debye^2, 1/s, cm/mol */
  double t[4];                /* transition moments, [idegI + 2*idegF] */
  double Elow, Eup;           /* E - ZPE of the initial and final level */
} or_line;

/* TROVE's scaled factorial and 3j symbol (trove_functions.cpp:322-399). */
double or_fakt(double a);
double or_three_j(int j1, int j2, int j3, int k1, int k2, int k3);
/* threej table (trove_functions.cpp:899-925); out has (jmax+1)^2*9 doubles,
   entries the reference leaves unset are written as 0. */
void or_precompute_threej(int jmax, double* out);

/* ijterms[iterm + g*Maxsymcoeffs] (trove_functions.cpp:927-966). */
void or_compute_ijterms(const or_basis* b, int nrep, int32_t* ijterms);

/* Symmetrised -> primitive (dipole_kernals.cu:38-71). */
void or_correlate(const or_basis* b, const int32_t* ijterms, int nrep, const int32_t* degen,
                  int ideg, int gamma, const double* vsym, double* vprim);

/* Half line strength with the flipped dipole (dipole_kernals.cu:162-227).
   mu is in record order; threej laid out as precompute_threej(jmax). */
void or_half_ls(const or_basis* bI, const or_basis* bF, int N, const double* mu,
                const double* threej, int jmax, const double* vprim, double* half_ls);

/* Accurate dot product (stand-in for cublasDdot, cuda_host.cu:1313). */
double or_dot(const double* x, const double* y, int n);

/* The driver loop of one reference run over jvals[0..1]
   (cuda_host.cu:1174-1477 with read_eigenvalues trove_functions.cpp:1075-1429).
   Lines are returned in (ilevelI, ilevelF) order of the energy-sorted level
   table; *out is malloc'ed (free with or_free).  Returns 0 or a negative error. */
int or_run(const or_job* job, or_line** out, size_t* nout);
void or_free(void* p);

/* Resolved ZPE of a job (read_eigenvalues first pass). */
double or_resolve_zpe(const or_job* job);

/* Filters of one level pair, ZPE taken as given: out = [energy_filter_lower(I),
   energy_filter_upper(F), intensity_filter(I,F)] (trove_functions.cpp:1432-1464). */
int or_filter_pair(const or_job* job, int jI, double EI, int gI, const int32_t* qI, int jF,
                   double EF, int gF, const int32_t* qF, int32_t* out, int32_t* igamma_pair);
/* degeneracy_filter (trove_functions.cpp:1495-1510). */
int or_degeneracy_filter(const or_job* job, int gI, int gF, int idegI, int idegF);

#ifdef __cplusplus
}
#endif
#endif
