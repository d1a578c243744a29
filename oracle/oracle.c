/*
 * CPU oracle for the line-intensity hot path (test infrastructure only; see
 * oracle.h).  Each function cites the reference file:line it restates.
 */
#include "oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_NINT(a) ((a) >= 0.0 ? (int)((a) + 0.5) : (int)((a)-0.5))

/* ---- Dot2 accumulator (Ogita, Rump, Oishi 2005) ------------------------- */
typedef struct {
  double s, c;
} dot2_acc;

static inline void dot2_add(dot2_acc* a, double x, double y) {
  double p = x * y;
  double ep = fma(x, y, -p); /* TwoProd error */
  double t = a->s + p;       /* TwoSum */
  double z = t - a->s;
  double es = (a->s - (t - z)) + (p - z);
  a->s = t;
  a->c += es + ep;
}
static inline double dot2_val(const dot2_acc* a) { return a->s + a->c; }

/* ---- 3j symbols --------------------------------------------------------- */

/* Scaled factorial a!/10^a as TROVE computes it (trove_functions.cpp:322-344):
   the running product of (a - i)/10 with the same operation order, so the
   3j values agree bit for bit with the reference's table. */
double or_fakt(double a) {
  double ax = a;
  double f = 1.0;
  if (fabs(ax) < 1e-24) return f;
  if (ax < 0.0) return NAN;
  int ic = OR_NINT(ax);
  ax = ax / 10.0;
  f = ax;
  for (int i = 1; i < ic; i++) f *= (ax - (double)i * 0.1);
  return f;
}

/* Wigner 3j (j1 j2 j3; k1 k2 k3) by the Racah sum over scaled factorials
   (trove_functions.cpp:349-399), including its phase (-1)^(j1-j2-k3). */
double or_three_j(int j1, int j2, int j3, int k1, int k2, int k3) {
  double a = j1, b = j2, c = j3, al = k1, be = k2, ga = k3;
  if (c > a + b) return 0.0;
  if (c < fabs(a - b)) return 0.0;
  if (a < 0.0 || b < 0.0 || c < 0.0) return 0.0;
  if (a < fabs(al) || b < fabs(be) || c < fabs(ga)) return 0.0;
  if (-1.0 * ga != al + be) return 0.0;

  double delta = sqrt(or_fakt(a + b - c) * or_fakt(a + c - b) * or_fakt(b + c - a) /
                      or_fakt(a + b + c + 1.0));
  double term1 = or_fakt(a + al) * or_fakt(a - al);
  double term2 = or_fakt(b - be) * or_fakt(b + be);
  double term3 = or_fakt(c + ga) * or_fakt(c - ga);
  double term = sqrt((2.0 * c + 1.0) * term1 * term2 * term3);

  double lo = a + be - c;
  if (b - c - al > lo) lo = b - c - al;
  if (0.0 > lo) lo = 0.0;
  double hi = a - al;
  if (b + be < hi) hi = b + be;
  if (a + b - c < hi) hi = a + b - c;
  int nmin = OR_NINT(lo), nmax = OR_NINT(hi);

  double summ = 0.0;
  for (int n = nmin; n <= nmax; n++) {
    double dn = (double)n;
    double t4 = or_fakt(a - al - dn) * or_fakt(c - b + al + dn);
    double t5 = or_fakt(b + be - dn) * or_fakt(c - a - be + dn);
    double t6 = or_fakt(dn) * or_fakt(a + b - c - dn);
    summ += pow(-1.0, n) / (t4 * t5 * t6);
  }
  double clebsh = delta * term * summ / sqrt(10.0);
  int iphase = OR_NINT(a - b - ga);
  double minus = (iphase % 2 == 0) ? 1.0 : -1.0;
  return minus * clebsh / sqrt(2.0 * c + 1.0);
}

/* threej[jI + kI*J1 + (dJ+1)*J1^2 + (dK+1)*3*J1^2], J1 = jmax+1
   (trove_functions.cpp:899-925).  Unset entries are zero here. */
void or_precompute_threej(int jmax, double* out) {
  int J1 = jmax + 1;
  memset(out, 0, sizeof(double) * (size_t)J1 * J1 * 9);
  for (int jI = 0; jI <= jmax; jI++)
    for (int jF = (jI - 1 > 0 ? jI - 1 : 0); jF <= (jI + 1 < jmax ? jI + 1 : jmax); jF++)
      for (int kI = 0; kI <= jI; kI++)
        for (int kF = (kI - 1 > 0 ? kI - 1 : 0); kF <= (kI + 1 < jF ? kI + 1 : jF); kF++)
          out[jI + kI * J1 + (jF - jI + 1) * J1 * J1 + (kF - kI + 1) * J1 * J1 * 3] =
              or_three_j(jI, 1, jF, kI, kF - kI, -kF);
}

/* Prefix sums of N per symmetry (trove_functions.cpp:927-966). */
void or_compute_ijterms(const or_basis* b, int nrep, int32_t* ijterms) {
  for (int g = 0; g < nrep; g++) {
    int n = 0;
    for (int it = 0; it < b->Maxsymcoeffs; it++) {
      ijterms[it + g * b->Maxsymcoeffs] = n;
      n += b->Nsym[g + it * nrep];
    }
  }
}

/* vprim[r] = sum_{i<nelem} vsym[iterm+i] * repres_g[(iterm+i) + ideg*Ntot + ib*degen*Ntot]
   (dipole_kernals.cu:38-71, the GPU indexing; not the CPU host_correlate_vectors). */
void or_correlate(const or_basis* b, const int32_t* ijterms, int nrep, const int32_t* degen,
                  int ideg, int gamma, const double* vsym, double* vprim) {
  int D = b->Maxcontracts;
  int Ntot = b->Ntotal[gamma];
  int sdeg = degen[gamma];
  const double* irr = b->repres[gamma];
  for (int r = 0; r < D; r++) {
    int irow = b->icontr2icase[r];
    int ib = b->icontr2icase[r + D];
    int iterm = ijterms[irow + gamma * b->Maxsymcoeffs];
    int nelem = b->Nsym[gamma + irow * nrep];
    dot2_acc acc = {0.0, 0.0};
    for (int i = 0; i < nelem; i++) {
      int s = iterm + i;
      dot2_add(&acc, vsym[s], irr[(size_t)s + (size_t)ideg * Ntot + (size_t)ib * sdeg * Ntot]);
    }
    vprim[r] = dot2_val(&acc);
  }
}

/* Half line strength (dipole_kernals.cu:162-227):
     h[rF] = (-1)^sigmaF * sum_{rI, |kI-kF|<=1} (-1)^(sigmaI+kI) * L * f3j * vI[rI] * s
   with sigma = (k mod 3)*tau, tau = ktau&1,
     kF == kI:           L = (tauF-tauI) * mu_z
     tauF != tauI:       L = (tauF-tauI)*(kF-kI) * mu_x
     otherwise:          L = -mu_y
   s = 1/sqrt(2) when kI != kF and kI*kF != 0, else 1, and the dipole read at
   the flipped position [icontrF + icontrI*N + c*N^2] = record mu_c(icontrI, icontrF).
   Terms with |kI-kF| > 1 are zero in the reference (multiplied by 0) and are
   skipped here. */
void or_half_ls(const or_basis* bI, const or_basis* bF, int N, const double* mu,
                const double* threej, int jmax, const double* vprim, double* half_ls) {
  const double sq2 = 1.0 / sqrt(2.0);
  const size_t N2 = (size_t)N * N;
  const int J1 = jmax + 1;
  const int jI = bI->jval, jF = bF->jval;
  const int DI = bI->Maxcontracts, DF = bF->Maxcontracts;
  for (int rF = 0; rF < DF; rF++) {
    int icF = bF->iroot_correlat_j0[rF];
    int tauF = bF->ktau[rF] & 1;
    int kF = bF->k[rF];
    int sigF = (kF % 3) * tauF;
    dot2_acc acc = {0.0, 0.0};
    for (int rI = 0; rI < DI; rI++) {
      int kI = bI->k[rI];
      if (abs(kI - kF) > 1) continue;
      int icI = bI->iroot_correlat_j0[rI];
      int tauI = bI->ktau[rI] & 1;
      int sigI = (kI % 3) * tauI;
      double sgnI = ((sigI + kI) & 1) ? -1.0 : 1.0;
      double f3j = threej[jI + kI * J1 + (jF - jI + 1) * J1 * J1 + (kF - kI + 1) * J1 * J1 * 3];
      int c;
      double L;
      if (kF == kI) {
        c = 2;
        L = (double)(tauF - tauI);
      } else if (tauF != tauI) {
        c = 0;
        L = (double)((tauF - tauI) * (kF - kI));
      } else {
        c = 1;
        L = -1.0;
      }
      double s = (kI != kF && kI * kF != 0) ? sq2 : 1.0;
      double m = mu[(size_t)c * N2 + (size_t)icI + (size_t)icF * N];
      double coef = sgnI * L * f3j * s;
      dot2_add(&acc, coef * m, vprim[rI]);
    }
    double sgnF = (sigF & 1) ? -1.0 : 1.0;
    half_ls[rF] = sgnF * dot2_val(&acc);
  }
}

double or_dot(const double* x, const double* y, int n) {
  dot2_acc acc = {0.0, 0.0};
  for (int i = 0; i < n; i++) dot2_add(&acc, x[i], y[i]);
  return dot2_val(&acc);
}

/* ---- Level table (trove_functions.cpp:1025-1028, 1075-1429) ------------- */

typedef struct {
  int jind, jval, gamma, rec, ndeg;
  double energy;
  const int32_t* quanta;
} or_level;

static int isym_do(const or_job* job, int g) { return !(job->gns[g] <= 0.00000001); }

static void eranges(const or_job* job, double er[2]) {
  er[0] = job->erange_lower[0] < job->erange_upper[0] ? job->erange_lower[0] : job->erange_upper[0];
  er[1] = job->erange_lower[1] > job->erange_upper[1] ? job->erange_lower[1] : job->erange_upper[1];
}

/* ZPE: while it is negative, every J=0, Gamma=0 record read replaces it
   (trove_functions.cpp:1200-1201); only files of enabled symmetries are read. */
double or_resolve_zpe(const or_job* job) {
  double zpe = job->ZPE;
  for (int i = 0; i < 2; i++) {
    if (job->jvals[i] != 0) continue;
    if (!isym_do(job, 0)) continue;
    const or_block* b = &job->blocks[i + 2 * 0];
    for (int r = 0; r < b->nvec; r++)
      if (zpe < 0) zpe = b->energies[r];
    break; /* the first pass reads jvals[0] before jvals[1]; one J=0 file */
  }
  return zpe;
}

static int cmp_level(const void* pa, const void* pb) {
  const or_level* a = (const or_level*)pa;
  const or_level* b = (const or_level*)pb;
  if (a->energy < b->energy) return -1;
  if (a->energy > b->energy) return 1;
  /* stable: keep the read order (jind, gamma, record) */
  if (a->jind != b->jind) return a->jind - b->jind;
  if (a->gamma != b->gamma) return a->gamma - b->gamma;
  return a->rec - b->rec;
}

/* ---- Filters (trove_functions.cpp:1432-1510) ---------------------------- */

typedef struct {
  const or_job* job;
  double zpe;
  int igamma_pair[16];
} or_ctx;

static int filt_lower(const or_ctx* x, int J, double E, const int32_t* q) {
  const or_job* job = x->job;
  for (int i = 0; i < job->nmodes; i++) {
    if (q[i + 1] < job->quanta_lower[i]) return 0;
    if (q[i + 1] > job->quanta_lower[job->nmodes + i]) return 0;
  }
  return J >= job->jvals[0] && J <= job->jvals[1] && (E - x->zpe) >= job->erange_lower[0] &&
         (E - x->zpe) <= job->erange_lower[1];
}

static int filt_upper(const or_ctx* x, int J, double E, const int32_t* q) {
  const or_job* job = x->job;
  for (int i = 0; i < job->nmodes; i++) {
    if (q[i + 1] < job->quanta_upper[i]) return 0;
    if (q[i + 1] > job->quanta_upper[job->nmodes + i]) return 0;
  }
  return J >= job->jvals[0] && J <= job->jvals[1] && (E - x->zpe) >= job->erange_upper[0] &&
         (E - x->zpe) <= job->erange_upper[1];
}

static int filt_intensity(const or_ctx* x, const or_level* I, const or_level* F) {
  const or_job* job = x->job;
  double nu = F->energy - I->energy;
  int passed = (job->gns[I->gamma] > 0.0) && (nu >= job->freq_window[0]) &&
               (nu <= job->freq_window[1]) && filt_lower(x, I->jval, I->energy, I->quanta) &&
               filt_upper(x, F->jval, F->energy, F->quanta);
  if (passed)
    passed = ((F->jval != job->jvals[0]) || (I->jval != job->jvals[0])) &&
             (job->isym_pairs[I->gamma] == job->isym_pairs[F->gamma]) &&
             (x->igamma_pair[I->gamma] == F->gamma) && (abs(F->jval - I->jval) <= 1) &&
             (I->jval + F->jval >= 1);
  return passed;
}

static int filt_degeneracy(const or_job* job, int gI, int gF, int idegI, int idegF) {
  if (job->degen[gI] == 1 || job->degen[gF] == 1) return 1;
  if (!job->reduced) return 1;
  if (job->sym_type == 2 || job->sym_type == 3) return (idegI == 1 && idegF == 0);
  return 1;
}

/* ---- Driver-loop arithmetic, two modes ---------------------------------- */
/* precise = 1 (the checker): every reduction in double-double.  The
   correlated vectors, the half line strength and the final dot carry a high
   and a low part, products of (hi + lo) operands are formed with TwoProd and
   accumulated with TwoSum (Dot2 with double-double inputs), so a transition
   moment is accurate to ~1e-30 of the sum of its terms' magnitudes and the
   relative error of a line measures the engine even where its moment is
   cancelled far below the terms.  precise = 0 (the port timed as the CPU
   baseline): the reference's own plain FP64 sums in its order. */

typedef struct {
  double s, c;
} dd_acc;

/* acc += (ah + al) * (bh + bl); al * bl is below 2^-106 of the term */
static inline void dd_add(dd_acc* a, double ah, double al, double bh, double bl) {
  double p = ah * bh;
  double ep = fma(ah, bh, -p) + (ah * bl + al * bh);
  double t = a->s + p;
  double z = t - a->s;
  double es = (a->s - (t - z)) + (p - z);
  a->s = t;
  a->c += es + ep;
}
static inline void dd_split(const dd_acc* a, double* hi, double* lo) {
  double h = a->s + a->c;
  *lo = a->c - (h - a->s);
  *hi = h;
}

/* correlate (dipole_kernals.cu:38-71) into hi/lo (lo = 0 in plain mode) */
static void corr_mode(const or_basis* b, const int32_t* ijterms, int nrep, const int32_t* degen,
                      int ideg, int gamma, const double* vsym, int precise, double* hi,
                      double* lo) {
  const int D = b->Maxcontracts;
  const int Ntot = b->Ntotal[gamma];
  const int sdeg = degen[gamma];
  const double* irr = b->repres[gamma];
  for (int r = 0; r < D; r++) {
    const int irow = b->icontr2icase[r];
    const int ib = b->icontr2icase[r + D];
    const int iterm = ijterms[irow + gamma * b->Maxsymcoeffs];
    const int nelem = b->Nsym[gamma + irow * nrep];
    const double* rr = irr + (size_t)ideg * Ntot + (size_t)ib * sdeg * Ntot;
    if (precise) {
      dd_acc acc = {0.0, 0.0};
      for (int i = 0; i < nelem; i++) dd_add(&acc, vsym[iterm + i], 0.0, rr[iterm + i], 0.0);
      dd_split(&acc, &hi[r], &lo[r]);
    } else {
      double acc = 0.0;
      for (int i = 0; i < nelem; i++) acc += vsym[iterm + i] * rr[iterm + i];
      hi[r] = acc;
      lo[r] = 0.0;
    }
  }
}

/* Roots of a basis grouped by k, ascending root index within each k. */
typedef struct {
  int kmax;
  int* ptr; /* [kmax+2] */
  int* idx; /* [D] */
} kgroups;

static void kgroups_build(const or_basis* b, kgroups* g) {
  const int D = b->Maxcontracts;
  int kmax = 0;
  for (int r = 0; r < D; r++)
    if (b->k[r] > kmax) kmax = b->k[r];
  g->kmax = kmax;
  g->ptr = (int*)calloc((size_t)kmax + 2, sizeof(int));
  g->idx = (int*)malloc(sizeof(int) * (size_t)(D > 0 ? D : 1));
  for (int r = 0; r < D; r++) g->ptr[b->k[r] + 1]++;
  for (int k = 0; k <= kmax; k++) g->ptr[k + 1] += g->ptr[k];
  int* fill = (int*)malloc(sizeof(int) * ((size_t)kmax + 1));
  for (int k = 0; k <= kmax; k++) fill[k] = g->ptr[k];
  for (int r = 0; r < D; r++) g->idx[fill[b->k[r]]++] = r;
  free(fill);
}
static void kgroups_free(kgroups* g) {
  free(g->ptr);
  free(g->idx);
}

/* Half line strength (dipole_kernals.cu:162-227) of one primitive initial
   vector into hi/lo, one final root per iteration (parallel over rF).  The
   reference's terms with |kI - kF| > 1 are exact zeros (multiplied by 0) and
   are skipped: the initial roots of kF-1, kF, kF+1 are visited in ascending
   root order, the reference's order, by a merge of the three k groups. */
static void half_ls_mode(const or_basis* bI, const kgroups* gI, const or_basis* bF, int N,
                         const double* mu, const double* threej, int jmax, const double* vh,
                         const double* vl, int precise, int nthreads, double* hh, double* hl) {
  const double sq2 = 1.0 / sqrt(2.0);
  const size_t N2 = (size_t)N * N;
  const int J1 = jmax + 1;
  const int jI = bI->jval, jF = bF->jval;
  const int DF = bF->Maxcontracts;
#pragma omp parallel for schedule(dynamic, 64) num_threads(nthreads)
  for (int rF = 0; rF < DF; rF++) {
    const int icF = bF->iroot_correlat_j0[rF];
    const int tauF = bF->ktau[rF] & 1;
    const int kF = bF->k[rF];
    const int sigF = (kF % 3) * tauF;
    int pos[3], end[3], ng = 0;
    for (int kI = kF - 1; kI <= kF + 1; kI++) {
      if (kI < 0 || kI > gI->kmax) continue;
      pos[ng] = gI->ptr[kI];
      end[ng] = gI->ptr[kI + 1];
      ng++;
    }
    dd_acc acc = {0.0, 0.0};
    double plain = 0.0;
    for (;;) {
      int best = -1, rI = 0;
      for (int q = 0; q < ng; q++)
        if (pos[q] < end[q] && (best < 0 || gI->idx[pos[q]] < rI)) {
          best = q;
          rI = gI->idx[pos[q]];
        }
      if (best < 0) break;
      pos[best]++;
      const int kI = bI->k[rI];
      const int icI = bI->iroot_correlat_j0[rI];
      const int tauI = bI->ktau[rI] & 1;
      const int sigI = (kI % 3) * tauI;
      const double sgnI = ((sigI + kI) & 1) ? -1.0 : 1.0;
      const double f3j =
          threej[jI + kI * J1 + (jF - jI + 1) * J1 * J1 + (kF - kI + 1) * J1 * J1 * 3];
      int c;
      double L;
      if (kF == kI) {
        c = 2;
        L = (double)(tauF - tauI);
      } else if (tauF != tauI) {
        c = 0;
        L = (double)((tauF - tauI) * (kF - kI));
      } else {
        c = 1;
        L = -1.0;
      }
      const double sc = (kI != kF && kI * kF != 0) ? sq2 : 1.0;
      const double m = mu[(size_t)c * N2 + (size_t)icI + (size_t)icF * N];
      const double coef = sgnI * L * f3j * sc;
      if (precise) {
        /* (coef * m) exactly as a pair, times vI = vh + vl */
        const double p = coef * m;
        const double pe = fma(coef, m, -p);
        dd_add(&acc, p, pe, vh[rI], vl[rI]);
      } else {
        plain += coef * m * vh[rI];
      }
    }
    const double sgnF = (sigF & 1) ? -1.0 : 1.0;
    if (precise) {
      double h, l;
      dd_split(&acc, &h, &l);
      hh[rF] = sgnF * h;
      hl[rF] = sgnF * l;
    } else {
      hh[rF] = sgnF * plain;
      hl[rF] = 0.0;
    }
  }
}

static double dot_mode(const double* xh, const double* xl, const double* yh, const double* yl,
                       int n, int precise) {
  if (precise) {
    dd_acc acc = {0.0, 0.0};
    for (int i = 0; i < n; i++) dd_add(&acc, xh[i], xl[i], yh[i], yl[i]);
    return acc.s + acc.c;
  }
  double acc = 0.0;
  for (int i = 0; i < n; i++) acc += xh[i] * yh[i];
  return acc;
}

/* ---- The driver loop (cuda_host.cu:1170-1477) --------------------------- */

int or_run(const or_job* job, or_line** out, size_t* nout) {
  *out = NULL;
  *nout = 0;
  if (job->nrep > 16) return -1;
  const int nrep = job->nrep;
  const int precise = job->precise;
#ifdef _OPENMP
  const int nth = job->nthreads > 0 ? job->nthreads : omp_get_max_threads();
#else
  const int nth = 1;
#endif
  or_ctx x;
  x.job = job;
  x.zpe = or_resolve_zpe(job);

  /* igamma pairs (trove_functions.cpp:1041-1072) */
  for (int gI = 0; gI < nrep; gI++) {
    int n = 0;
    x.igamma_pair[gI] = gI;
    for (int gF = 0; gF < nrep; gF++)
      if (gI != gF && job->isym_pairs[gI] == job->isym_pairs[gF]) {
        x.igamma_pair[gI] = gF;
        if (++n > 1) return -2;
      }
    if (job->gns[gI] != job->gns[x.igamma_pair[gI]]) return -3;
  }

  /* level table */
  double er[2];
  eranges(job, er);
  size_t cap = 0;
  for (int i = 0; i < 2; i++)
    for (int g = 0; g < nrep; g++) cap += (size_t)job->blocks[i + 2 * g].nvec;
  or_level* lv = (or_level*)malloc(sizeof(or_level) * (cap ? cap : 1));
  int nl = 0;
  for (int i = 0; i < 2; i++)
    for (int g = 0; g < nrep; g++) {
      if (!isym_do(job, g)) continue;
      const or_block* b = &job->blocks[i + 2 * g];
      for (int r = 0; r < b->nvec; r++) {
        double E = b->energies[r];
        if (!((E - x.zpe) >= er[0] && (E - x.zpe) <= er[1])) continue;
        or_level L = {i, job->jvals[i], g, r, job->degen[g], E,
                      b->quanta + (size_t)r * (job->nmodes + 1)};
        lv[nl++] = L;
      }
    }
  qsort(lv, (size_t)nl, sizeof(or_level), cmp_level);

  /* symmetric-index offsets and k groups per basis */
  int32_t* ijt[2];
  kgroups kg[2];
  for (int i = 0; i < 2; i++) {
    ijt[i] = (int32_t*)malloc(sizeof(int32_t) * (size_t)job->basis[i].Maxsymcoeffs * nrep);
    or_compute_ijterms(&job->basis[i], nrep, ijt[i]);
    kgroups_build(&job->basis[i], &kg[i]);
  }
  int jmax = job->jvals[0] > job->jvals[1] ? job->jvals[0] : job->jvals[1];
  double* threej = (double*)malloc(sizeof(double) * (size_t)(jmax + 1) * (jmax + 1) * 9);
  or_precompute_threej(jmax, threej);

  const int dimenmax = job->basis[0].Maxcontracts > job->basis[1].Maxcontracts
                           ? job->basis[0].Maxcontracts
                           : job->basis[1].Maxcontracts;
  int maxdeg = 1;
  for (int g = 0; g < nrep; g++)
    if (job->degen[g] > maxdeg) maxdeg = job->degen[g];

  /* initial levels that pass the lower filter */
  int* inits = (int*)malloc(sizeof(int) * (size_t)(nl ? nl : 1));
  int ninit = 0;
  for (int li = 0; li < nl; li++)
    if (filt_lower(&x, lv[li].jval, lv[li].energy, lv[li].quanta)) inits[ninit++] = li;

  /* correlated final vectors: cached for every level when they fit in 2 GiB
     and more than one initial level uses them, else formed per use */
  const size_t corr_elems = (size_t)nl * maxdeg * dimenmax;
  const int cache_corr = ninit > 1 && corr_elems * 2 * sizeof(double) <= ((size_t)2 << 30);
  double* corr_h = NULL;
  double* corr_l = NULL;
  if (cache_corr) {
    corr_h = (double*)malloc(sizeof(double) * corr_elems + 8);
    corr_l = (double*)malloc(sizeof(double) * corr_elems + 8);
#pragma omp parallel for schedule(dynamic, 4) num_threads(nth)
    for (int l = 0; l < nl; l++) {
      const or_level* F = &lv[l];
      const or_block* b = &job->blocks[F->jind + 2 * F->gamma];
      for (int d = 0; d < F->ndeg; d++) {
        const size_t o = ((size_t)l * maxdeg + d) * dimenmax;
        corr_mode(&job->basis[F->jind], ijt[F->jind], nrep, job->degen, d, F->gamma,
                  b->vecs + (size_t)F->rec * b->nsize, precise, corr_h + o, corr_l + o);
      }
    }
  }

  /* constants (cuda_host.cu:12-18, 1170) */
  const double pi = 4.0 * atan2(1.0, 1.0);
  const double planck = 6.62606896e-27, avogno = 6.0221415e23, vellgt = 2.99792458e10,
               boltz = 1.380658e-16;
  const double A_coef_s_1 = 64.0 * pow(10.0, -36.0) * pow(pi, 4.0) / (3.0 * 6.62606896 * pow(10.0, -27.0));
  const double intens_cm_mol =
      8.0 * pow(10.0, -36.0) * pow(pi, 3.0) * avogno / (3.0 * planck * vellgt);
  const double beta = planck * vellgt / (boltz * job->temperature);

  /* one line slot per final level of the current initial level */
  or_line* row = (or_line*)malloc(sizeof(or_line) * (size_t)(nl ? nl : 1));
  char* keep = (char*)malloc((size_t)(nl ? nl : 1));
  size_t total = 0, acap = 1024;
  or_line* all = (or_line*)malloc(sizeof(or_line) * acap);
  double* vh = (double*)malloc(sizeof(double) * dimenmax);
  double* vl = (double*)malloc(sizeof(double) * dimenmax);
  double* hh = (double*)malloc(sizeof(double) * 2 * maxdeg * dimenmax);
  double* hl = (double*)malloc(sizeof(double) * 2 * maxdeg * dimenmax);
  int err = 0;

  for (int ii = 0; ii < ninit; ii++) {
    const or_level* I = &lv[inits[ii]];
    const or_block* bI = &job->blocks[I->jind + 2 * I->gamma];
    const double* vecI = bI->vecs + (size_t)I->rec * bI->nsize;
    const int gFt = x.igamma_pair[I->gamma];
    int have[2][2] = {{0, 0}, {0, 0}};
    for (int indF = 0; indF < 2; indF++) {
      const int jF = job->jvals[indF];
      /* indF_filter (trove_functions.cpp:1476-1493) */
      int any = 0;
      for (int lf = 0; lf < nl && !any; lf++)
        if (lv[lf].jval == jF && filt_intensity(&x, I, &lv[lf])) any = 1;
      if (!any) continue;
      for (int d = 0; d < I->ndeg; d++) {
        if (!filt_degeneracy(job, I->gamma, gFt, d, 0)) continue;
        corr_mode(&job->basis[I->jind], ijt[I->jind], nrep, job->degen, d, I->gamma, vecI,
                  precise, vh, vl);
        const size_t o = ((size_t)indF + 2 * d) * dimenmax;
        half_ls_mode(&job->basis[I->jind], &kg[I->jind], &job->basis[indF], job->N, job->mu,
                     threej, jmax, vh, vl, precise, nth, hh + o, hl + o);
        have[indF][d] = 1;
      }
    }
#pragma omp parallel num_threads(nth)
    {
      double* fh = NULL;
      double* fl = NULL;
      if (!cache_corr) {
        fh = (double*)malloc(sizeof(double) * dimenmax);
        fl = (double*)malloc(sizeof(double) * dimenmax);
      }
#pragma omp for schedule(dynamic, 16)
      for (int lf = 0; lf < nl; lf++) {
        keep[lf] = 0;
        const or_level* F = &lv[lf];
        if (!filt_upper(&x, F->jval, F->energy, F->quanta)) continue;
        if (!filt_intensity(&x, I, F)) continue;
        double t[4] = {0.0, 0.0, 0.0, 0.0};
        const int dimenF = job->basis[F->jind].Maxcontracts;
        const or_block* bF = &job->blocks[F->jind + 2 * F->gamma];
        for (int dF = 0; dF < F->ndeg; dF++) {
          if (job->reduced && dF != 0) continue;
          const double* ch;
          const double* cl;
          if (cache_corr) {
            ch = corr_h + ((size_t)lf * maxdeg + dF) * dimenmax;
            cl = corr_l + ((size_t)lf * maxdeg + dF) * dimenmax;
          } else {
            corr_mode(&job->basis[F->jind], ijt[F->jind], nrep, job->degen, dF, F->gamma,
                      bF->vecs + (size_t)F->rec * bF->nsize, precise, fh, fl);
            ch = fh;
            cl = fl;
          }
          for (int dI = 0; dI < I->ndeg; dI++) {
            if (!filt_degeneracy(job, I->gamma, F->gamma, dI, dF)) continue;
            if (!have[F->jind][dI]) {
#pragma omp atomic write
              err = -4;
              continue;
            }
            const size_t o = ((size_t)F->jind + 2 * dI) * dimenmax;
            t[dI + 2 * dF] = dot_mode(ch, cl, hh + o, hl + o, dimenF, precise);
          }
        }
        /* epilogue (cuda_host.cu:1388-1407) */
        double ls = 0.0;
        for (int dF = 0; dF < F->ndeg; dF++)
          for (int dI = 0; dI < I->ndeg; dI++) ls += t[dI + 2 * dF] * t[dI + 2 * dF];
        ls /= (double)I->ndeg;
        if (job->reduced && F->ndeg != 1 && I->ndeg != 1) ls *= (double)I->ndeg;
        const double nu = F->energy - I->energy;
        const double anu = fabs(nu);
        const double boltz_fc =
            anu * exp(-(I->energy - x.zpe) * beta) * (1.0 - exp(-anu * beta)) / job->q_stat;
        const double A = A_coef_s_1 * (double)(2 * I->jval + 1) * ls * pow(anu, 3);
        const double S = ls * job->gns[I->gamma] * (double)((2 * I->jval + 1) * (2 * F->jval + 1));
        const double In = S * intens_cm_mol * boltz_fc;
        if (!(S >= job->thresh_linestrength)) continue;
        if (!(In / avogno >= job->thresh_intensity)) continue;
        or_line* o = &row[lf];
        o->jI = I->jval;
        o->gammaI = I->gamma;
        o->recI = I->rec;
        o->jF = F->jval;
        o->gammaF = F->gamma;
        o->recF = F->rec;
        o->ndegI = I->ndeg;
        o->ndegF = F->ndeg;
        o->nu = nu;
        o->S = S;
        o->A = A;
        o->I = In;
        memcpy(o->t, t, sizeof(t));
        o->Elow = I->energy - x.zpe;
        o->Eup = F->energy - x.zpe;
        keep[lf] = 1;
      }
      free(fh);
      free(fl);
    }
    for (int lf = 0; lf < nl; lf++) {
      if (!keep[lf]) continue;
      if (total == acap) {
        acap *= 2;
        all = (or_line*)realloc(all, sizeof(or_line) * acap);
      }
      all[total++] = row[lf];
    }
  }

  free(row);
  free(keep);
  free(vh);
  free(vl);
  free(hh);
  free(hl);
  free(inits);
  free(corr_h);
  free(corr_l);
  free(threej);
  for (int i = 0; i < 2; i++) {
    free(ijt[i]);
    kgroups_free(&kg[i]);
  }
  free(lv);
  if (err) {
    free(all);
    return err;
  }
  *out = all;
  *nout = total;
  return 0;
}

void or_free(void* p) { free(p); }

/* Filters of one level pair with the job's ZPE as given (for pinning against
   the reference's energy_filter_lower/upper and intensity_filter). */
int or_filter_pair(const or_job* job, int jI, double EI, int gI, const int32_t* qI, int jF,
                   double EF, int gF, const int32_t* qF, int32_t* out, int32_t* igamma_pair) {
  or_ctx x;
  x.job = job;
  x.zpe = job->ZPE;
  for (int a = 0; a < job->nrep; a++) {
    int n = 0;
    x.igamma_pair[a] = a;
    for (int b = 0; b < job->nrep; b++)
      if (a != b && job->isym_pairs[a] == job->isym_pairs[b]) {
        x.igamma_pair[a] = b;
        if (++n > 1) return -2;
      }
    igamma_pair[a] = x.igamma_pair[a];
  }
  or_level I = {0, jI, gI, 0, job->degen[gI], EI, qI};
  or_level F = {0, jF, gF, 0, job->degen[gF], EF, qF};
  out[0] = filt_lower(&x, jI, EI, qI);
  out[1] = filt_upper(&x, jF, EF, qF);
  out[2] = filt_intensity(&x, &I, &F);
  return 0;
}

int or_degeneracy_filter(const or_job* job, int gI, int gF, int idegI, int idegF) {
  return filt_degeneracy(job, gI, gF, idegI, idegF);
}
