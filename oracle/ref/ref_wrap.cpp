// C entry points over the reference's own CPU functions and kernel bodies,
// compiled from the reference sources by oracle/build_ref.sh into
// oracle/_ref/libref.so.  Used only to pin the oracle (test infrastructure);
// the kernels run as host loops over thread ids (see inc/cuda_runtime_api.h).
#include <cuda_runtime_api.h>  // the host stand-in in oracle/ref/inc

#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <new>
#include <algorithm>
#include <vector>
#include <unistd.h>

#include "cuda_objects.cuh"
#include "dipole_kernals.cuh"
#include "fields.h"
#include "trove_functions.h"
#include "../oracle.h"

// Zero-filled array allocations: the reference's threej table leaves slots it
// never reads with a nonzero weight uninitialised; zeroing keeps its kernels'
// 0*slot products finite.
void* operator new[](size_t n) {
  void* p = std::calloc(n ? n : 1, 1);
  if (!p) throw std::bad_alloc();
  return p;
}
void operator delete[](void* p) noexcept { std::free(p); }
void operator delete[](void* p, size_t) noexcept { std::free(p); }

gi_ref_dim3 blockIdx, blockDim, threadIdx, gridDim;
double s[1];  // backs the reference's `extern __shared__ double s[]` (unused kernels)
extern intensity_info int_info;

namespace {

struct RefBasis {
  cuda_bset_contrT c;
  TO_bset_contrT t;
  std::vector<double*> irr;
  std::vector<int*> nper;
  int* ijterms = nullptr;
};

void make_basis(const or_basis* b, int nrep, RefBasis& rb) {
  std::memset(&rb.c, 0, sizeof(rb.c));
  std::memset(&rb.t, 0, sizeof(rb.t));
  rb.t.jval = b->jval;
  rb.t.Maxsymcoeffs = b->Maxsymcoeffs;
  rb.t.Maxcontracts = b->Maxcontracts;
  rb.t.max_deg_size = b->max_deg_size;
  rb.t.mat_size = b->mat_size;
  rb.t.irr = new TO_PTrepresT[nrep];
  rb.nper.resize(nrep);
  for (int g = 0; g < nrep; g++) {
    rb.nper[g] = new int[b->Maxsymcoeffs];
    for (int ic = 0; ic < b->Maxsymcoeffs; ic++) rb.nper[g][ic] = b->Nsym[g + ic * nrep];
    rb.t.irr[g].N = rb.nper[g];
    rb.t.irr[g].repres = const_cast<double*>(b->repres[g]);
  }
  compute_ijterms(rb.t, &rb.ijterms, nrep);
  rb.irr.resize(nrep);
  for (int g = 0; g < nrep; g++) rb.irr[g] = const_cast<double*>(b->repres[g]);
  rb.c.jval = b->jval;
  rb.c.Maxsymcoeffs = b->Maxsymcoeffs;
  rb.c.max_deg_size = b->max_deg_size;
  rb.c.Maxcontracts = b->Maxcontracts;
  rb.c.icontr2icase = const_cast<int*>(b->icontr2icase);
  rb.c.iroot_correlat_j0 = const_cast<int*>(b->iroot_correlat_j0);
  rb.c.k = const_cast<int*>(b->k);
  rb.c.ktau = const_cast<int*>(b->ktau);
  rb.c.irr_repres = rb.irr.data();
  rb.c.N = const_cast<int*>(b->Nsym);
  rb.c.Ntotal = const_cast<int*>(b->Ntotal);
  rb.c.ijterms = rb.ijterms;
}

void free_basis(RefBasis& rb, int nrep) {
  for (int g = 0; g < nrep; g++) delete[] rb.nper[g];
  delete[] rb.t.irr;
  delete[] rb.ijterms;
}

void set_info(int nrep, const int* degen, int jmax, int N, int dimenmax) {
  intensity_info ii;
  ii.sym_nrepres = nrep;
  ii.sym_degen = const_cast<int*>(degen);
  ii.jmax = jmax + 1;  // as cuda_host.cu:913
  ii.dip_stride_1 = N;
  ii.dip_stride_2 = N * N;
  ii.dimenmax = dimenmax;
  ii.sq2 = 1.0 / std::sqrt(2.0);
  copy_intensity_info(&ii);
}

void one_thread_grid() {
  blockIdx = {0, 0, 0};
  threadIdx = {0, 0, 0};
  blockDim = {1, 1, 1};
  gridDim = {1, 1, 1};
}

void fill_job(const or_job* j, FintensityJob& f, std::vector<int*>& keep) {
  std::memset((void*)&f, 0, sizeof(f));
  f.ZPE = j->ZPE;
  for (int i = 0; i < 2; i++) {
    f.erange_lower[i] = j->erange_lower[i];
    f.erange_upper[i] = j->erange_upper[i];
    f.freq_window[i] = j->freq_window[i];
    f.jvals[i] = j->jvals[i];
  }
  f.erange[0] = std::min(f.erange_lower[0], f.erange_upper[0]);
  f.erange[1] = std::max(f.erange_lower[1], f.erange_upper[1]);
  f.q_stat = j->q_stat;
  f.temperature = j->temperature;
  f.molec.nmodes = j->nmodes;
  f.molec.sym_nrepres = j->nrep;
  f.molec.sym_degen = const_cast<int*>(j->degen);
  f.molec.sym_type = j->sym_type;
  f.gns = const_cast<double*>(j->gns);
  f.isym_pairs = const_cast<int*>(j->isym_pairs);
  f.igamma_pair = new int[j->nrep];
  keep.push_back(f.igamma_pair);
  f.reduced = j->reduced != 0;
  f.quanta_lower = new int*[2];
  f.quanta_upper = new int*[2];
  for (int i = 0; i < 2; i++) {
    f.quanta_lower[i] = const_cast<int*>(j->quanta_lower) + i * j->nmodes;
    f.quanta_upper[i] = const_cast<int*>(j->quanta_upper) + i * j->nmodes;
  }
  f.isym_do = new bool[j->nrep];
  for (int g = 0; g < j->nrep; g++) f.isym_do[g] = !(j->gns[g] <= 0.00000001);
}

void drop_job(FintensityJob& f, std::vector<int*>& keep) {
  for (int* p : keep) delete[] p;
  delete[] f.quanta_lower;
  delete[] f.quanta_upper;
  delete[] f.isym_do;
}

}  // namespace

extern "C" {

double ref_fakt(double a) { return fakt(a); }
double ref_three_j(int j1, int j2, int j3, int k1, int k2, int k3) {
  return three_j(j1, j2, j3, k1, k2, k3);
}

void ref_precompute_threej(int jmax, double* out) {
  double* t = nullptr;
  precompute_threej(&t, jmax);
  std::memcpy(out, t, sizeof(double) * (size_t)(jmax + 1) * (jmax + 1) * 9);
  delete[] t;
}

void ref_compute_ijterms(const or_basis* b, int nrep, int* out) {
  RefBasis rb;
  make_basis(b, nrep, rb);
  std::memcpy(out, rb.ijterms, sizeof(int) * (size_t)b->Maxsymcoeffs * nrep);
  free_basis(rb, nrep);
}

// device_correlate_vectors (dipole_kernals.cu:38-71), one host call per root.
void ref_correlate(const or_basis* b, int nrep, const int* degen, int ideg, int gamma,
                   const double* vsym, double* vprim) {
  RefBasis rb;
  make_basis(b, nrep, rb);
  set_info(nrep, degen, b->jval, 1, b->Maxcontracts);
  one_thread_grid();
  for (int r = 0; r < b->Maxcontracts; r++) {
    blockIdx.x = (unsigned)r;
    device_correlate_vectors(&rb.c, ideg, gamma, vsym, vprim);
  }
  free_basis(rb, nrep);
}

// device_compute_1st_half_ls_flipped_dipole (dipole_kernals.cu:162-227) with a
// one-thread grid, so its grid-stride loop covers every final root.
// dip_flipped is the layout read_dipole_flipped produces.
void ref_half_ls_flipped(const or_basis* bI, const or_basis* bF, int nrep, const int* degen,
                         int N, const double* dip_flipped, int jmax, const double* threej,
                         const double* vprim, double* half_ls) {
  RefBasis ri, rf;
  make_basis(bI, nrep, ri);
  make_basis(bF, nrep, rf);
  int dmax = std::max(bI->Maxcontracts, bF->Maxcontracts);
  set_info(nrep, degen, jmax, N, dmax);
  one_thread_grid();
  device_compute_1st_half_ls_flipped_dipole(&ri.c, &rf.c, const_cast<double*>(dip_flipped),
                                            const_cast<double*>(vprim),
                                            const_cast<double*>(threej), half_ls);
  free_basis(ri, nrep);
  free_basis(rf, nrep);
}

// read_dipole_flipped (trove_functions.cpp:113-205) on a j0_extfield.chk in dir.
int ref_read_dipole_flipped(const char* dir, int N, double* out) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir) != 0) return -2;
  TO_bset_contrT b;
  std::memset((void*)&b, 0, sizeof(b));
  b.Maxcontracts = N;
  double* d = nullptr;
  size_t sz = 0;
  read_dipole_flipped(b, &d, sz);
  int rc = chdir(cwd);
  (void)rc;
  std::memcpy(out, d, sz);
  delete[] d;
  return (int)(sz / sizeof(double));
}

// Filters (trove_functions.cpp:1041-1072, 1432-1510) on one level pair.
// Writes [lower(I), upper(F), intensity(I,F), indF-free] and igamma pairs.
int ref_filters(const or_job* j, int jI, double EI, int gI, const int* qI, int jF, double EF,
                int gF, const int* qF, int* out, int* igamma_pair) {
  FintensityJob f;
  std::vector<int*> keep;
  fill_job(j, f, keep);
  find_igamma_pair(f);
  for (int g = 0; g < j->nrep; g++) igamma_pair[g] = f.igamma_pair[g];
  out[0] = energy_filter_lower(f, jI, EI, const_cast<int*>(qI));
  out[1] = energy_filter_upper(f, jF, EF, const_cast<int*>(qF));
  out[2] = intensity_filter(f, jI, jF, EI, EF, gI, gF, const_cast<int*>(qI), const_cast<int*>(qF));
  drop_job(f, keep);
  return 0;
}

int ref_degeneracy_filter(const or_job* j, int gI, int gF, int idegI, int idegF) {
  FintensityJob f;
  std::vector<int*> keep;
  fill_job(j, f, keep);
  int r = degeneracy_filter(f, gI, gF, idegI, idegF);
  drop_job(f, keep);
  return r;
}


// bset_contr_factory + correlate_index (trove_functions.cpp:401-858) on the
// j0eigen_quanta files in dir.  dims receives {D, ncase, max_deg, mat_size,
// nclasses}; with k == NULL only dims and Ntotal (when given) are filled.
int ref_read_quanta(const char* dir, int J, int nrep, const int* degen, int* dims, int* k,
                    int* ktau, int* iroot, int* icontr2icase, int* Nsym, int* Ntotal,
                    double** repres) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir) != 0) return -2;
  TO_bset_contrT b0, b;
  std::memset((void*)&b0, 0, sizeof(b0));
  std::memset((void*)&b, 0, sizeof(b));
  bset_contr_factory(&b0, 0, const_cast<int*>(degen), nrep);
  TO_bset_contrT* t = &b0;
  if (J != 0) {
    bset_contr_factory(&b, J, const_cast<int*>(degen), nrep);
    t = &b;
  }
  correlate_index(b0, *t);
  int rc = chdir(cwd);
  (void)rc;
  const int D = t->Maxcontracts;
  dims[0] = D;
  dims[1] = t->Maxsymcoeffs;
  dims[2] = t->max_deg_size;
  dims[3] = t->mat_size;
  dims[4] = t->Nclasses;
  if (Ntotal) std::memcpy(Ntotal, t->Ntotal, sizeof(int) * nrep);
  if (!k) return 0;
  std::memcpy(k, t->k, sizeof(int) * D);
  std::memcpy(ktau, t->ktau, sizeof(int) * D);
  std::memcpy(iroot, t->iroot_correlat_j0, sizeof(int) * D);
  std::memcpy(icontr2icase, t->icontr2icase, sizeof(int) * 2 * D);
  for (int g = 0; g < nrep; g++) {
    for (int ic = 0; ic < t->Maxsymcoeffs; ic++) Nsym[g + ic * nrep] = t->irr[g].N[ic];
    std::memcpy(repres[g], t->irr[g].repres,
                sizeof(double) * (size_t)t->Ntotal[g] * degen[g] * t->mat_size);
  }
  return 0;
}

// read_eigenvalues (trove_functions.cpp:1075-1429) for jvals (j0, j1) on the
// descr files in dir; the level fields as ref_level records.
struct ref_level {
  int jval, igamma, ilevel, ndeg, irec0, irec1, krot, taurot;
  double energy;
  int quanta[17], normal[17], cgamma[17];
};

int ref_read_levels(const char* dir, int j0, int j1, int sym_type, int nrep, const int* degen,
                    int nmodes, int nclasses, double zpe, double elow, double ehigh,
                    const double* gns, int maxcontracts, int cap, ref_level* out) {
  char cwd[4096];
  if (!getcwd(cwd, sizeof(cwd))) return -1;
  if (chdir(dir) != 0) return -2;
  FintensityJob f;
  std::memset((void*)&f, 0, sizeof(f));
  f.jvals[0] = j0;
  f.jvals[1] = j1;
  f.ZPE = zpe;
  f.erange[0] = elow;
  f.erange[1] = ehigh;
  f.molec.nmodes = nmodes;
  f.molec.nclasses = nclasses;
  f.molec.sym_nrepres = nrep;
  f.molec.sym_degen = const_cast<int*>(degen);
  f.molec.sym_type = sym_type;
  f.molec.c_sym = new char*[nrep];
  for (int g = 0; g < nrep; g++) {
    f.molec.c_sym[g] = new char[4];
    std::snprintf(f.molec.c_sym[g], 4, "%d", g);
  }
  f.isym_do = new bool[nrep];
  for (int g = 0; g < nrep; g++) f.isym_do[g] = gns[g] > 0.00000001;
  for (int i = 0; i < 3; i++) {
    f.bset_contr[i].Maxcontracts = maxcontracts;
    f.bset_contr[i].nsize = new int[nrep];
  }
  read_eigenvalues(f);
  int rc = chdir(cwd);
  (void)rc;
  const int n = std::min(cap, f.Neigenlevels);
  for (int i = 0; i < n; i++) {
    const TO_PTeigen& e = f.eigen[i];
    ref_level& r = out[i];
    std::memset(&r, 0, sizeof(r));
    r.jval = e.jval;
    r.igamma = e.igamma;
    r.ilevel = e.ilevel;
    r.ndeg = e.ndeg;
    r.irec0 = e.irec[0];
    r.irec1 = e.ndeg > 1 ? e.irec[1] : 0;
    r.krot = e.krot;
    r.taurot = e.taurot;
    r.energy = e.energy;
    for (int q = 0; q <= nmodes && q < 17; q++) {
      r.quanta[q] = e.quanta[q];
      r.normal[q] = e.normal[q];
    }
    for (int q = 0; q <= nclasses && q < 17; q++) r.cgamma[q] = std::atoi(e.cgamma[q]);
  }
  return f.Neigenlevels;
}

}  // extern "C"
