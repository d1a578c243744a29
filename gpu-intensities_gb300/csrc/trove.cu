// TROVE job files and the reference's text interfaces (host code only):
//   - the input deck (fields.cpp:11-282),
//   - the checkpoints: j0_extfield.chk (Fortran records of the vibrational
//     dipole, trove_functions.cpp:113-205), j0eigen_quanta<J>.chk (the
//     contracted basis, bset_contr_factory and correlate_index,
//     trove_functions.cpp:401-858), j0eigen_descr<J>_<G>.chk (levels,
//     read_eigenvalues, trove_functions.cpp:1075-1429) and
//     j0eigen_vectors<J>_<G>.chk (raw eigenvector records, cuda_host.cu:1196),
//   - the printed line list (cuda_host.cu:1444-1473),
//   - the partition function the reference takes as QSTAT from the deck.
// File formats and field meanings follow the reference readers so that the
// same files give the same tables; the parsing code is this project's.
#include <cuda_runtime.h>

#include <algorithm>
#include <cctype>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <string>
#include <unordered_map>
#include <vector>

#include "engine.h"

namespace gi {
namespace {

// ------------------------------------------------------------------ errors
gi_status set_err(char* err, size_t cap, gi_status s, const char* fmt, ...) {
  if (err && cap) {
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(err, cap, fmt, ap);
    va_end(ap);
  }
  return s;
}

std::string path_of(const char* dir, const std::string& name) {
  std::string d = dir ? dir : ".";
  if (d.empty()) d = ".";
  if (d.back() != '/') d += '/';
  return d + name;
}

std::string trimmed(const std::string& s) {
  size_t a = 0, b = s.size();
  while (a < b && std::isspace((unsigned char)s[a])) a++;
  while (b > a && std::isspace((unsigned char)s[b - 1])) b--;
  return s.substr(a, b - a);
}

// Whitespace-separated numbers of one text line, read like the reference's
// strtol(.., 0) / strtod chains.
struct Tok {
  const char* p;
  explicit Tok(const std::string& s) : p(s.c_str()) {}
  long i() {
    char* e = nullptr;
    const long v = std::strtol(p, &e, 0);
    p = e;
    return v;
  }
  double d() {
    char* e = nullptr;
    const double v = std::strtod(p, &e);
    p = e;
    return v;
  }
};

struct LineReader {
  FILE* f = nullptr;
  explicit LineReader(const std::string& path) { f = std::fopen(path.c_str(), "r"); }
  ~LineReader() {
    if (f) std::fclose(f);
  }
  bool get(std::string& line) {
    line.clear();
    if (!f) return false;
    int c;
    bool any = false;
    while ((c = std::fgetc(f)) != EOF) {
      any = true;
      if (c == '\n') break;
      line.push_back((char)c);
    }
    if (!line.empty() && line.back() == '\r') line.pop_back();
    return any;
  }
};

// ------------------------------------------------------------------ symmetry
struct SymInfo {
  int type;
  const char* name;
  std::vector<int> degen;
  std::vector<const char*> labels;
};
const SymInfo* sym_info(int type) {
  static const SymInfo tab[] = {
      {1, "C2V(M)", {1, 1, 1, 1}, {"A1", "A2", "B1", "B2"}},
      {2, "C3V(M)", {1, 1, 2}, {"A1", "A2", "E"}},
      {3, "D3H(M)", {1, 1, 2, 1, 1, 2}, {"A1'", "A2'", "E'", "A1\"", "A2\"", "E\""}},
  };
  for (const SymInfo& s : tab)
    if (s.type == type) return &s;
  return nullptr;
}

// ------------------------------------------------------------------ basis file
struct BasisFile {
  int J = 0, ncases = 0, nlambdas = 0, ncontr = 0, nclasses = 0;
  int rot_ncases = 0, rot_nlambdas = 0, mat_size = 0;
  std::vector<int> cspace;                 // [(nclasses+1) * ncases], 0-based
  std::vector<int> size1;                  // lambdas of each case
  std::vector<std::vector<int>> icoeffs;   // per case [(nclasses+1) * size1], 0-based
  std::vector<int> icontr2icase;           // [2 * ncontr]
  std::vector<int> icase2icontr;           // [ncases * nlambdas]
  std::vector<int> rot_k, rot_tau;         // [rot_ncases * rot_nlambdas]
  std::vector<int> Ntotal, Nsym;           // Nsym[g + case * nrep]
  std::vector<std::vector<double>> repres; // per gamma [Ntotal * degen * mat_size]
  std::vector<int> k, ktau, iroot;         // correlate_index
};

// bset_contr_factory (trove_functions.cpp:401-679)
gi_status read_basis_file(const char* dir, int J, const SymInfo& sym, BasisFile& b, char* err,
                          size_t cap) {
  char name[64];
  std::snprintf(name, sizeof(name), "j0eigen_quanta%d.chk", J);
  const std::string path = path_of(dir, name);
  LineReader in(path);
  if (!in.f) return set_err(err, cap, GI_ERR_NOTFOUND, "cannot open %s", path.c_str());
  std::string line;
  in.get(line);
  if (trimmed(line) != "Start Primitive basis set")
    return set_err(err, cap, GI_ERR_ARG, "%s: bad header", path.c_str());
  in.get(line);
  {
    Tok t(line);
    b.ncases = (int)t.i();
    b.nlambdas = (int)t.i();
    b.ncontr = (int)t.i();
    b.nclasses = (int)t.i();
  }
  b.J = J;
  const int nc1 = b.nclasses + 1;
  if (b.ncases <= 0 || b.nlambdas <= 0 || b.ncontr <= 0 || b.nclasses < 0)
    return set_err(err, cap, GI_ERR_ARG, "%s: bad sizes", path.c_str());
  b.cspace.assign((size_t)nc1 * b.ncases, 0);
  b.size1.assign(b.ncases, 0);
  b.icoeffs.assign(b.ncases, {});
  b.icontr2icase.assign(2 * (size_t)b.ncontr, 0);
  b.icase2icontr.assign((size_t)b.ncases * b.nlambdas, -1);
  int icontr = 0;
  for (int icase = 0; icase < b.ncases; icase++) {
    if (!in.get(line)) return set_err(err, cap, GI_ERR_ARG, "%s: truncated", path.c_str());
    Tok t(line);
    const int nl = (int)t.i();
    if (nl < 0 || nl > b.nlambdas)
      return set_err(err, cap, GI_ERR_ARG, "%s: case %d has %d lambdas", path.c_str(), icase, nl);
    for (int i = 0; i < nc1; i++) b.cspace[i + (size_t)icase * nc1] = (int)t.i() - 1;
    b.size1[icase] = nl;
    b.icoeffs[icase].assign((size_t)nc1 * nl, 0);
    for (int il = 0; il < nl; il++) {
      if (!in.get(line)) return set_err(err, cap, GI_ERR_ARG, "%s: truncated", path.c_str());
      Tok u(line);
      const int iroot = (int)u.i() - 1;
      for (int i = 0; i < nc1; i++) b.icoeffs[icase][i + (size_t)il * nc1] = (int)u.i() - 1;
      if (iroot != icontr || icontr >= b.ncontr)
        return set_err(err, cap, GI_ERR_ARG, "%s: wrong indexing icontr=%d iroot=%d",
                       path.c_str(), icontr, iroot);
      b.icontr2icase[icontr] = icase;
      b.icontr2icase[icontr + b.ncontr] = il;
      b.icase2icontr[icase + (size_t)il * b.ncases] = icontr;
      icontr++;
    }
  }
  if (icontr != b.ncontr) return set_err(err, cap, GI_ERR_ARG, "%s: wrong indexing", path.c_str());
  in.get(line);
  {
    Tok t(line);
    b.rot_ncases = (int)t.i();
    b.rot_nlambdas = (int)t.i();
  }
  if (b.rot_ncases <= 0 || b.rot_nlambdas <= 0)
    return set_err(err, cap, GI_ERR_ARG, "%s: bad rotational index sizes", path.c_str());
  b.rot_k.assign((size_t)b.rot_ncases * b.rot_nlambdas, 0);
  b.rot_tau.assign((size_t)b.rot_ncases * b.rot_nlambdas, 0);
  bool ended = false;
  while (in.get(line)) {
    if (trimmed(line) == "End Primitive basis set") {
      ended = true;
      break;
    }
    Tok t(line);
    const int ic = (int)t.i() - 1, il = (int)t.i() - 1;
    t.i();  // j
    const int kk = (int)t.i(), tau = (int)t.i();
    if (ic < 0 || ic >= b.rot_ncases || il < 0 || il >= b.rot_nlambdas)
      return set_err(err, cap, GI_ERR_ARG, "%s: rotational index out of range", path.c_str());
    b.rot_k[ic + (size_t)il * b.rot_ncases] = kk;
    b.rot_tau[ic + (size_t)il * b.rot_ncases] = tau;
  }
  if (!ended) return set_err(err, cap, GI_ERR_ARG, "%s: no basis footer", path.c_str());
  in.get(line);
  if (trimmed(line) != "Start irreducible transformation")
    return set_err(err, cap, GI_ERR_ARG, "%s: wrong sym-footer", path.c_str());
  const int nrep = (int)sym.degen.size();
  in.get(line);
  b.mat_size = (int)Tok(line).i();
  in.get(line);
  {
    Tok t(line);
    b.Ntotal.assign(nrep, 0);
    for (int g = 0; g < nrep; g++) b.Ntotal[g] = (int)t.i();
  }
  if (b.mat_size <= 0) return set_err(err, cap, GI_ERR_ARG, "%s: bad mat_size", path.c_str());
  b.Nsym.assign((size_t)nrep * b.ncases, 0);
  b.repres.assign(nrep, {});
  for (int g = 0; g < nrep; g++) {
    for (int ic = 0; ic < b.ncases; ic++) {
      if (!in.get(line)) return set_err(err, cap, GI_ERR_ARG, "%s: truncated N", path.c_str());
      b.Nsym[g + (size_t)ic * nrep] = (int)Tok(line).i();
    }
    const int nt = std::max(b.Ntotal[g], 0), dg = sym.degen[g];
    b.repres[g].assign((size_t)nt * dg * b.mat_size, 0.0);
    for (int s = 0; s < nt; s++)
      for (int d = 0; d < dg; d++) {
        if (!in.get(line)) return set_err(err, cap, GI_ERR_ARG, "%s: truncated repres", path.c_str());
        Tok t(line);
        for (int i = 0; i < b.mat_size; i++)
          b.repres[g][s + (size_t)d * nt + (size_t)i * nt * dg] = t.d();
      }
  }
  in.get(line);
  if (trimmed(line) != "End irreducible transformation")
    return set_err(err, cap, GI_ERR_ARG, "%s: wrong irrep-footer", path.c_str());
  return GI_OK;
}

// correlate_index (trove_functions.cpp:681-858): the J=0 contracted function
// with the same vibrational labels, and k, 2k+tau of every root.  The first
// match in the reference's (jcase, jlambda) order wins.
gi_status correlate(const BasisFile& b0, BasisFile& b, char* err, size_t cap) {
  if (b0.J != 0) return set_err(err, cap, GI_ERR_ARG, "correlation needs the J=0 basis");
  if (b0.nclasses != b.nclasses)
    return set_err(err, cap, GI_ERR_ARG, "Nclasses differ between J=0 and J=%d", b.J);
  const int nc = b.nclasses, nc1 = nc + 1;
  auto key_of = [nc](const int* cs, const int* ic) {
    std::string k;
    k.reserve(8 * (size_t)nc);
    for (int i = 1; i <= nc; i++) k.append((const char*)&cs[i], sizeof(int));
    for (int i = 1; i <= nc; i++) k.append((const char*)&ic[i], sizeof(int));
    return k;
  };
  std::unordered_map<std::string, int> j0;
  for (int jc = 0; jc < b0.ncases; jc++)
    for (int jl = 0; jl < b0.size1[jc]; jl++) {
      const std::string k = key_of(&b0.cspace[(size_t)jc * nc1], &b0.icoeffs[jc][(size_t)jl * nc1]);
      if (!j0.count(k)) j0[k] = b0.icase2icontr[jc + (size_t)jl * b0.ncases];
    }
  b.iroot.assign(b.ncontr, 0);
  b.k.assign(b.ncontr, 0);
  b.ktau.assign(b.ncontr, 0);
  for (int r = 0; r < b.ncontr; r++) {
    const int ic = b.icontr2icase[r], il = b.icontr2icase[r + b.ncontr];
    auto it = j0.find(key_of(&b.cspace[(size_t)ic * nc1], &b.icoeffs[ic][(size_t)il * nc1]));
    if (it == j0.end())
      return set_err(err, cap, GI_ERR_ARG, "no J=0 correlation for J=%d case %d lambda %d", b.J,
                     ic, il);
    if (it->second < 0 || it->second >= b0.ncontr)
      return set_err(err, cap, GI_ERR_ARG, "root correlation out of range for J=%d", b.J);
    b.iroot[r] = it->second;
    const int ilevel = b.cspace[(size_t)ic * nc1];
    const int ideg = b.icoeffs[ic][(size_t)il * nc1];
    const size_t ri = (size_t)ilevel + (size_t)ideg * b.rot_ncases;
    if (ilevel < 0 || ideg < 0 || ri >= b.rot_k.size())
      return set_err(err, cap, GI_ERR_ARG, "rotational index out of range for J=%d", b.J);
    b.k[r] = b.rot_k[ri];
    b.ktau[r] = 2 * b.rot_k[ri] + b.rot_tau[ri];
  }
  return GI_OK;
}

// ------------------------------------------------------------------ dipole
bool read_record(FILE* f, std::vector<char>& out) {
  int32_t n = 0, m = 0;
  if (std::fread(&n, 4, 1, f) != 1 || n < 0) return false;
  out.resize((size_t)n);
  if (n && std::fread(out.data(), 1, (size_t)n, f) != (size_t)n) return false;
  if (std::fread(&m, 4, 1, f) != 1 || m != n) return false;
  return true;
}

// read_dipole_flipped (trove_functions.cpp:113-205) without the flip: the
// records as stored, mu_c(i, f) at c*N*N + i + f*N.
gi_status read_dipole(const char* dir, int N, double* mu, char* err, size_t cap) {
  const std::string path = path_of(dir, "j0_extfield.chk");
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return set_err(err, cap, GI_ERR_NOTFOUND, "cannot open %s", path.c_str());
  std::vector<char> rec;
  gi_status st = GI_OK;
  auto bad = [&](const char* what) {
    st = set_err(err, cap, GI_ERR_ARG, "%s: %s", path.c_str(), what);
  };
  if (!read_record(f, rec) || rec.size() < 20 || std::memcmp(rec.data(), "Start external field", 20))
    bad("bogus header");
  int32_t n = 0;
  if (st == GI_OK && (!read_record(f, rec) || rec.size() != 4)) bad("bad size record");
  if (st == GI_OK) {
    std::memcpy(&n, rec.data(), 4);
    if (n != N) st = set_err(err, cap, GI_ERR_ARG, "%s: N=%d, the J=0 basis has %d", path.c_str(), n, N);
  }
  for (int c = 0; c < 3 && st == GI_OK; c++) {
    int32_t imu = 0;
    if (!read_record(f, rec) || rec.size() != 4) {
      bad("bad component record");
      break;
    }
    std::memcpy(&imu, rec.data(), 4);
    if (imu != c + 1) {
      bad("bogus imu");
      break;
    }
    if (!read_record(f, rec) || rec.size() != sizeof(double) * (size_t)N * N) {
      bad("bad matrix record");
      break;
    }
    if (mu) std::memcpy(mu + (size_t)c * N * N, rec.data(), rec.size());
  }
  if (st == GI_OK && (!read_record(f, rec) || rec.size() < 18 ||
                      std::memcmp(rec.data(), "End external field", 18)))
    bad("bogus footer");
  std::fclose(f);
  return st;
}

// ------------------------------------------------------------------ levels
// read_eigenvalues (trove_functions.cpp:1075-1429) for one (J, gamma) file:
// every ideg = 1 line is a level, in file order, with the records of all its
// degenerate components.
gi_status read_descr(const char* dir, int J, int gamma, int sym_type, int nmodes, int nclasses,
                     std::vector<gi_trove_level>& out, int* dim_basis, char* err, size_t cap) {
  char name[64];
  std::snprintf(name, sizeof(name), "j0eigen_descr%d_%d.chk", J, gamma + 1);
  const std::string path = path_of(dir, name);
  LineReader in(path);
  if (!in.f) return set_err(err, cap, GI_ERR_NOTFOUND, "cannot open %s", path.c_str());
  const SymInfo* sym = sym_info(sym_type);
  if (!sym || gamma < 0 || gamma >= (int)sym->degen.size())
    return set_err(err, cap, GI_ERR_ARG, "bad symmetry or gamma");
  if (nmodes < 0 || nmodes >= GI_TROVE_MAXQ || nclasses < 0 || nclasses >= GI_TROVE_MAXQ)
    return set_err(err, cap, GI_ERR_ARG, "nmodes/nclasses beyond %d", GI_TROVE_MAXQ - 1);
  std::string line;
  bool found = false;
  while (in.get(line))
    if (trimmed(line) == "Start Quantum numbers and energies") {
      found = true;
      break;
    }
  if (!found) return set_err(err, cap, GI_ERR_ARG, "%s: malformed descr file", path.c_str());
  in.get(line);
  in.get(line);
  in.get(line);
  {
    Tok t(line);
    t.i();  // nroots
    *dim_basis = (int)t.i();
  }
  // ktau_rot: level quanta(0) -> (k, tau) (trove_functions.cpp:1278-1298)
  auto krot_of = [J](int q0, int* krot, int* taurot) {
    if (q0 <= 0) {
      *krot = 0;
      *taurot = J % 2;
    } else {
      *krot = (q0 + 1) / 2;
      *taurot = (q0 + 1) % 2;
    }
  };
  std::map<int, size_t> by_level;  // ilevel -> index in out
  out.clear();
  while (in.get(line)) {
    if (trimmed(line) == "End Quantum numbers and energies") break;
    if (trimmed(line).empty()) continue;
    Tok t(line);
    const int irec = (int)t.i();
    const int igamma = (int)t.i();
    if (igamma != gamma + 1)
      return set_err(err, cap, GI_ERR_ARG, "%s: gamma %d in the file of gamma %d", path.c_str(),
                     igamma, gamma + 1);
    const int ilevel = (int)t.i() - 1;
    const int ideg = (int)t.i();
    const double energy = t.d();
    if (ideg < 1 || ideg > sym->degen[gamma])
      return set_err(err, cap, GI_ERR_ARG, "%s: ideg %d", path.c_str(), ideg);
    if (ideg == 1) {
      gi_trove_level L;
      std::memset(&L, 0, sizeof(L));
      L.irec[0] = irec;
      L.ilevel = ilevel;
      L.ndeg = sym->degen[gamma];
      L.energy = energy;
      for (int q = 0; q <= nmodes; q++) L.quanta[q] = (int32_t)t.i();
      L.large_coef = (int32_t)t.i();
      for (int q = 0; q <= nclasses; q++) L.cgamma[q] = (int32_t)t.i() - 1;
      for (int q = 0; q <= nmodes; q++) L.normal[q] = (int32_t)t.i();
      krot_of(L.quanta[0], &L.krot, &L.taurot);
      by_level[ilevel] = out.size();
      out.push_back(L);
    } else {
      auto it = by_level.find(ilevel);
      if (it == by_level.end())
        return set_err(err, cap, GI_ERR_ARG, "%s: component %d before its level", path.c_str(), ideg);
      out[it->second].irec[ideg - 1] = irec;
    }
  }
  return GI_OK;
}

gi_status read_vectors(const char* dir, int J, int gamma, int nsize,
                       const std::vector<gi_trove_level>& lv, double* out, char* err, size_t cap) {
  char name[64];
  std::snprintf(name, sizeof(name), "j0eigen_vectors%d_%d.chk", J, gamma + 1);
  const std::string path = path_of(dir, name);
  FILE* f = std::fopen(path.c_str(), "rb");
  if (!f) return set_err(err, cap, GI_ERR_NOTFOUND, "cannot open %s", path.c_str());
  gi_status st = GI_OK;
  for (size_t i = 0; i < lv.size() && st == GI_OK; i++) {
    const long long off = (long long)(lv[i].irec[0] - 1) * nsize * (long long)sizeof(double);
    if (lv[i].irec[0] < 1 || std::fseek(f, (long)off, SEEK_SET) != 0 ||
        std::fread(out + i * (size_t)nsize, sizeof(double), (size_t)nsize, f) != (size_t)nsize)
      st = set_err(err, cap, GI_ERR_ARG, "%s: cannot read record %d", path.c_str(), lv[i].irec[0]);
  }
  std::fclose(f);
  return st;
}

// ------------------------------------------------------------------ deck
// fields.cpp:145-282: read_fields (NMODES, SYMGROUP, INTENSITY) and
// read_intensities (until END).  Upper-cased, the first "(...)" of an
// intensity line removed, tokens split at blanks and commas.
std::vector<std::string> tokens(std::string line, bool strip_paren) {
  if (strip_paren) {
    const size_t a = line.find('('), b = line.find(')');
    if (a != std::string::npos) line.erase(a, (b == std::string::npos ? line.size() : b + 1) - a);
  }
  for (char& ch : line) ch = (char)std::toupper((unsigned char)ch);
  std::vector<std::string> t;
  std::string cur;
  for (char ch : line) {
    if (ch == ' ' || ch == ',' || ch == '\t') {
      if (!cur.empty()) t.push_back(cur);
      cur.clear();
    } else {
      cur.push_back(ch);
    }
  }
  if (!cur.empty()) t.push_back(cur);
  return t;
}

}  // namespace

// ------------------------------------------------------------------ context
// TROVE descriptors of the loaded levels, kept for the printed line list.
struct TroveMeta {
  int nmodes = 0, nclasses = 0;
  std::map<std::pair<int, int>, std::vector<gi_trove_level>> levels;  // (J, gamma) -> block rows
};

void trove_meta_release(Ctx* c) {
  delete c->trove;
  c->trove = nullptr;
}

}  // namespace gi

using namespace gi;

extern "C" {

gi_status gi_deck_parse(const char* text, gi_deck* d, char* err, size_t cap) {
  if (!text || !d) return GI_ERR_ARG;
  std::memset(d, 0, sizeof(*d));
  gi_params& p = d->params;
  // windows wide open and thresholds off unless the deck sets them (the
  // reference leaves them uninitialised)
  p.temperature = 296.0;
  p.q_stat = 1.0;
  p.erange_lower[0] = p.erange_upper[0] = -1e300;
  p.erange_lower[1] = p.erange_upper[1] = 1e300;
  p.freq_window[0] = -1e300;
  p.freq_window[1] = 1e300;
  for (int g = 0; g < GI_MAX_REP; g++) p.gns[g] = 1.0;
  for (int i = 0; i < GI_MAX_MODES; i++) {
    p.quanta_lower[0][i] = p.quanta_upper[0][i] = -1000000000;
    p.quanta_lower[1][i] = p.quanta_upper[1][i] = 1000000000;
  }
  d->sym_type = 0;
  int nrep = 0;
  bool in_intensity = false;
  const char* s = text;
  while (*s) {
    const char* e = std::strchr(s, '\n');
    std::string line(s, e ? (size_t)(e - s) : std::strlen(s));
    s = e ? e + 1 : s + line.size();
    std::vector<std::string> t = tokens(line, in_intensity);
    if (t.empty()) continue;
    auto num = [&](size_t i, double* v) {
      if (i >= t.size()) return false;
      char* end = nullptr;
      *v = std::strtod(t[i].c_str(), &end);
      return end != t[i].c_str();
    };
    auto inum = [&](size_t i, int* v) {
      if (i >= t.size()) return false;
      char* end = nullptr;
      *v = (int)std::strtol(t[i].c_str(), &end, 0);
      return end != t[i].c_str();
    };
    if (!in_intensity) {
      if (t[0] == "NMODES") {
        if (!inum(1, &d->nmodes) || d->nmodes < 0 || d->nmodes > GI_MAX_MODES)
          return set_err(err, cap, GI_ERR_ARG, "NMODES: bad value");
        p.nmodes = d->nmodes;
      } else if (t[0] == "SYMGROUP") {
        if (t.size() < 2) return set_err(err, cap, GI_ERR_ARG, "SYMGROUP: missing name");
        for (int ty = 1; ty <= 3; ty++)
          if (t[1] == sym_info(ty)->name) d->sym_type = ty;
        if (!d->sym_type) return set_err(err, cap, GI_ERR_ARG, "symmetry %s not implemented", t[1].c_str());
        nrep = (int)sym_info(d->sym_type)->degen.size();
      } else if (t[0] == "INTENSITY") {
        in_intensity = true;
      }
      continue;
    }
    const std::string& k = t[0];
    bool ok = true;
    if (k == "END") {
      in_intensity = false;
    } else if (k == "TEMPERATURE") {
      ok = num(1, &p.temperature);
    } else if (k == "QSTAT") {
      ok = num(1, &p.q_stat);
    } else if (k == "ZPE") {
      ok = num(1, &p.ZPE);
    } else if (k == "J") {
      ok = inum(1, &d->jvals[0]) && inum(2, &d->jvals[1]);
    } else if (k == "FREQ-WINDOW") {
      ok = num(1, &p.freq_window[0]) && num(2, &p.freq_window[1]);
    } else if (k == "ENERGY") {
      for (size_t i = 1; i < t.size() && ok; i++) {
        if (t[i] == "LOW") {
          ok = num(i + 1, &p.erange_lower[0]) && num(i + 2, &p.erange_lower[1]);
          i += 2;
        } else if (t[i] == "UPPER") {
          ok = num(i + 1, &p.erange_upper[0]) && num(i + 2, &p.erange_upper[1]);
          i += 2;
        }
      }
    } else if (k == "GNS") {
      if (!nrep) return set_err(err, cap, GI_ERR_STATE, "GNS before SYMGROUP");
      for (int g = 0; g < nrep && ok; g++) ok = num(1 + g, &p.gns[g]);
    } else if (k == "SELECTION") {
      if (!nrep) return set_err(err, cap, GI_ERR_STATE, "SELECTION before SYMGROUP");
      for (int g = 0; g < nrep && ok; g++) ok = inum(1 + g, &p.isym_pairs[g]);
    } else if (k == "THRESH_LINE") {
      ok = num(1, &p.thresh_linestrength);
    } else if (k == "V") {
      int q = 0;
      ok = inum(1, &q) && q >= 1 && q <= GI_MAX_MODES;
      for (size_t i = 2; i < t.size() && ok; i++) {
        if (t[i] == "LOWER") {
          ok = inum(i + 1, &p.quanta_lower[0][q - 1]) && inum(i + 2, &p.quanta_lower[1][q - 1]);
          i += 2;
        } else if (t[i] == "UPPER") {
          ok = inum(i + 1, &p.quanta_upper[0][q - 1]) && inum(i + 2, &p.quanta_upper[1][q - 1]);
          i += 2;
        }
      }
    } else if (k == "SYMMETRY") {
      if (t.size() > 1 && t[1] == "REDUCED") p.reduced = 1;
    }
    if (!ok) return set_err(err, cap, GI_ERR_ARG, "deck: bad value in \"%s\"", line.c_str());
  }
  if (!d->sym_type) return set_err(err, cap, GI_ERR_ARG, "deck: no SYMGROUP");
  return GI_OK;
}

gi_status gi_trove_read_basis(const char* dir, int J, int sym_type, int32_t* dims, int32_t* k,
                              int32_t* ktau, int32_t* iroot, int32_t* icontr2icase, int32_t* Nsym,
                              int32_t* Ntotal, double* const* repres, char* err, size_t cap) {
  const SymInfo* sym = sym_info(sym_type);
  if (!sym || J < 0 || !dims) return set_err(err, cap, GI_ERR_ARG, "bad arguments");
  BasisFile b0, b;
  gi_status st = read_basis_file(dir, 0, *sym, b0, err, cap);
  if (st != GI_OK) return st;
  if (J == 0) {
    b = b0;
  } else {
    st = read_basis_file(dir, J, *sym, b, err, cap);
    if (st != GI_OK) return st;
  }
  st = correlate(b0, b, err, cap);
  if (st != GI_OK) return st;
  const int nrep = (int)sym->degen.size();
  dims[0] = b.ncontr;
  dims[1] = b.ncases;
  dims[2] = b.nlambdas;
  dims[3] = b.mat_size;
  dims[4] = b.nclasses;
  dims[5] = b0.ncontr;
  if (k) std::copy(b.k.begin(), b.k.end(), k);
  if (ktau) std::copy(b.ktau.begin(), b.ktau.end(), ktau);
  if (iroot) std::copy(b.iroot.begin(), b.iroot.end(), iroot);
  if (icontr2icase) std::copy(b.icontr2icase.begin(), b.icontr2icase.end(), icontr2icase);
  if (Nsym) std::copy(b.Nsym.begin(), b.Nsym.end(), Nsym);
  if (Ntotal) std::copy(b.Ntotal.begin(), b.Ntotal.end(), Ntotal);
  if (repres)
    for (int g = 0; g < nrep; g++)
      if (repres[g]) std::copy(b.repres[g].begin(), b.repres[g].end(), repres[g]);
  return GI_OK;
}

gi_status gi_trove_read_dipole(const char* dir, int N, double* mu, char* err, size_t cap) {
  if (N <= 0) return set_err(err, cap, GI_ERR_ARG, "bad N");
  return read_dipole(dir, N, mu, err, cap);
}

gi_status gi_trove_read_levels(const char* dir, int J, int gamma, int sym_type, int nmodes,
                               int nclasses, int32_t* n, int32_t* dim_basis, gi_trove_level* out,
                               int32_t cap_levels, char* err, size_t cap) {
  if (!n || !dim_basis) return set_err(err, cap, GI_ERR_ARG, "bad arguments");
  std::vector<gi_trove_level> lv;
  int dim = 0;
  gi_status st = read_descr(dir, J, gamma, sym_type, nmodes, nclasses, lv, &dim, err, cap);
  if (st != GI_OK) return st;
  *n = (int32_t)lv.size();
  *dim_basis = dim;
  if (out) std::copy(lv.begin(), lv.begin() + std::min<size_t>(lv.size(), (size_t)std::max(cap_levels, 0)), out);
  return GI_OK;
}

gi_status gi_load_trove(gi_ctx* h, const char* dir, const gi_deck* d, int flags) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !d) return GI_ERR_ARG;
  if (c->server) return fail(c, GI_ERR_STATE, "gi_load_trove while serving");
  const SymInfo* sym = sym_info(d->sym_type);
  if (!sym) return fail(c, GI_ERR_ARG, "deck symmetry %d not implemented", d->sym_type);
  char err[512] = {0};
  const int nrep = (int)sym->degen.size();
  std::vector<int> jlist;
  if (flags & GI_TROVE_ALL_J) {
    for (int J = d->jvals[0]; J <= d->jvals[1]; J++) jlist.push_back(J);
  } else {
    jlist.push_back(d->jvals[0]);
    if (d->jvals[1] != d->jvals[0]) jlist.push_back(d->jvals[1]);
  }
  if (jlist.empty() || jlist.front() < 0) return fail(c, GI_ERR_ARG, "deck: bad J values");
  gi_status st = gi_set_symmetry(h, d->sym_type);
  if (st != GI_OK) return st;
  gi_params p = d->params;
  if (c->have_params) {  // keep the context's precision choice
    p.precision = c->params.precision;
    p.split_slices = c->params.split_slices;
  }
  st = gi_set_params(h, &p);
  if (st != GI_OK) return st;
  // bases (J = 0 first: it defines the vibrational functions)
  BasisFile b0;
  st = read_basis_file(dir, 0, *sym, b0, err, sizeof(err));
  if (st != GI_OK) return fail(c, st, "%s", err);
  const int N = b0.ncontr;
  for (int J : jlist) {
    BasisFile b;
    if (J == 0) {
      b = b0;
    } else {
      st = read_basis_file(dir, J, *sym, b, err, sizeof(err));
      if (st != GI_OK) return fail(c, st, "%s", err);
    }
    st = correlate(b0, b, err, sizeof(err));
    if (st != GI_OK) return fail(c, st, "%s", err);
    std::vector<const double*> rep(nrep);
    for (int g = 0; g < nrep; g++) rep[g] = b.repres[g].data();
    st = gi_set_basis(h, J, b.ncontr, b.ncases, b.nlambdas, b.mat_size, b.icontr2icase.data(),
                      b.iroot.data(), b.k.data(), b.ktau.data(), b.Nsym.data(), b.Ntotal.data(),
                      rep.data());
    if (st != GI_OK) return st;
  }
  // dipole (record order); kept in host memory and streamed when asked or
  // when its padded copy would take more than half of the device (the
  // reference splits it above 5 GiB, cuda_host.cu:858-867)
  {
    const size_t bytes = sizeof(double) * 3 * (size_t)N * N;
    bool streamed = (flags & GI_TROVE_STREAM_DIPOLE) != 0;
    size_t free_b = 0, total_b = 0;
    cudaSetDevice(c->device);
    if (!streamed && cudaMemGetInfo(&free_b, &total_b) == cudaSuccess &&
        sizeof(double) * 3.0 * N * round_up(N, 64) > 0.5 * (double)total_b)
      streamed = true;
    if (streamed) {
      double* pinned = nullptr;
      GI_CUDA(c, cudaMallocHost(&pinned, bytes));
      st = read_dipole(dir, N, pinned, err, sizeof(err));
      if (st != GI_OK) {
        cudaFreeHost(pinned);
        return fail(c, st, "%s", err);
      }
      st = dipole_stream_adopt(c, N, pinned, 0);
    } else {
      std::vector<double> mu((size_t)3 * N * N);
      st = read_dipole(dir, N, mu.data(), err, sizeof(err));
      if (st != GI_OK) return fail(c, st, "%s", err);
      st = gi_set_dipole(h, N, mu.data());
    }
    if (st != GI_OK) return st;
  }
  // blocks: one row per level of every symmetry with g_ns > 0
  TroveMeta* meta = new TroveMeta();
  meta->nmodes = d->nmodes;
  meta->nclasses = b0.nclasses;
  for (int J : jlist)
    for (int g = 0; g < nrep; g++) {
      if (!(p.gns[g] > 0.00000001)) continue;
      std::vector<gi_trove_level> lv;
      int dim = 0;
      st = read_descr(dir, J, g, d->sym_type, d->nmodes, b0.nclasses, lv, &dim, err, sizeof(err));
      if (st != GI_OK) {
        delete meta;
        return fail(c, st, "%s", err);
      }
      const int nsize = c->bases[J]->Ntotal[g];
      if (!lv.empty() && dim != nsize) {
        delete meta;
        return fail(c, GI_ERR_ARG, "J=%d gamma=%d: descr dim_basis %d != Ntotal %d", J, g + 1, dim,
                    nsize);
      }
      std::vector<double> vecs((size_t)lv.size() * std::max(nsize, 1));
      if (!lv.empty()) {
        st = read_vectors(dir, J, g, nsize, lv, vecs.data(), err, sizeof(err));
        if (st != GI_OK) {
          delete meta;
          return fail(c, st, "%s", err);
        }
      }
      std::vector<double> energies(lv.size());
      std::vector<int32_t> quanta(lv.size() * (size_t)(d->nmodes + 1));
      for (size_t i = 0; i < lv.size(); i++) {
        energies[i] = lv[i].energy;
        for (int q = 0; q <= d->nmodes; q++) quanta[i * (d->nmodes + 1) + q] = lv[i].quanta[q];
      }
      st = gi_set_block(h, J, g, lv.empty() ? 0 : nsize, (int)lv.size(), vecs.data(),
                        energies.data(), quanta.data());
      if (st != GI_OK) {
        delete meta;
        return st;
      }
      meta->levels[{J, g}] = std::move(lv);
    }
  trove_meta_release(c);
  c->trove = meta;
  return GI_OK;
}

// Q = sum over the loaded levels of g_ns (2J+1) ndeg exp(-c2 (E - ZPE) / T),
// c2 = h c / k (the first radiation constant's partner, in cm K).
gi_status gi_partition_function(gi_ctx* h, double temperature, double* q) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || !q || !(temperature > 0)) return GI_ERR_ARG;
  if (!c->have_params) return fail(c, GI_ERR_STATE, "gi_set_params not called");
  double zpe = c->params.ZPE;
  auto it0 = c->blocks.find({0, 0});
  if (zpe < 0 && it0 != c->blocks.end() && !it0->second->energies.empty())
    zpe = it0->second->energies[0];
  const double sum = partition_sum(c, temperature, zpe);
  *q = sum;
  return GI_OK;
}

// The printed layout of one line (cuda_host.cu:1444-1473): the reference's
// printf sequence, field by field, appended to s.
static void format_line_text(const gi_line_text& f, std::string& s) {
  char tmp[128];
  const int dj = f.jF - f.jI;
  const char* br = dj == 0 ? "Q" : (dj == 1 ? "R" : "P");
  std::snprintf(tmp, sizeof(tmp), "%4i %4s   <-%4i %4s   %1s  %11.4f <- %11.4f %11.4f  ( %3s %3i ) ( ",
                f.jF, f.symF, f.jI, f.symI, br, f.eF, f.eI, std::fabs(f.nu), f.cgF[0], f.krotF);
  s += tmp;
  for (int i = 1; i <= f.nclasses; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3s", f.cgF[i]);
    s += tmp;
  }
  s += " ";
  for (int i = 1; i <= f.nmodes; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3i", f.quantaF[i]);
    s += tmp;
  }
  std::snprintf(tmp, sizeof(tmp), " ) <- ( %3s %3i ) ( ", f.cgI[0], f.krotI);
  s += tmp;
  for (int i = 1; i <= f.nclasses; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3s", f.cgI[i]);
    s += tmp;
  }
  s += " ";
  for (int i = 1; i <= f.nmodes; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3i", f.quantaI[i]);
    s += tmp;
  }
  std::snprintf(tmp, sizeof(tmp), ")  %16.8e %16.8e %16.8e   %6i <- %6i %8i %8i ( ", f.S, f.A,
                f.I, f.ilevelF + 1, f.ilevelI + 1, 0, 0);
  s += tmp;
  for (int i = 1; i <= f.nmodes; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3i", f.normalF[i]);
    s += tmp;
  }
  s += " ) <-  ( ";
  for (int i = 1; i <= f.nmodes; i++) {
    std::snprintf(tmp, sizeof(tmp), " %3i", f.normalI[i]);
    s += tmp;
  }
  s += " ) ";
  for (int dF = 0; dF < f.ndegF; dF++)
    for (int dI = 0; dI < f.ndegI; dI++) {
      std::snprintf(tmp, sizeof(tmp), " %16.9e", f.t[dI + 2 * dF]);
      s += tmp;
    }
  s += "\n";
}

gi_status gi_format_line_text(const gi_line_text* f, char* buf, size_t cap, size_t* used) {
  if (!f || !used || f->nclasses < 0 || f->nclasses >= GI_TROVE_MAXQ || f->nmodes < 0 ||
      f->nmodes >= GI_TROVE_MAXQ || f->ndegF < 1 || f->ndegF > 2 || f->ndegI < 1 || f->ndegI > 2 ||
      !f->symF || !f->symI)
    return GI_ERR_ARG;
  for (int q = 0; q <= f->nclasses; q++)
    if (!f->cgF[q] || !f->cgI[q]) return GI_ERR_ARG;
  std::string s;
  format_line_text(*f, s);
  *used = s.size();
  if (buf && cap) {
    const size_t n = std::min(cap - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
    if (s.size() >= cap) return GI_ERR_ARG;
  }
  return GI_OK;
}

// One line of the reference's list (cuda_host.cu:1444-1473) for each line of
// the last gi_run, "\n"-terminated.  The level descriptors come from
// gi_load_trove; levels loaded otherwise print their symmetry as the class
// labels, their quanta as normal-mode quanta and their record as level index.
gi_status gi_format_lines(gi_ctx* h, int64_t offset, int64_t count, char* buf, size_t cap,
                          size_t* used) {
  Ctx* c = reinterpret_cast<Ctx*>(h);
  if (!c || offset < 0 || count < 0 || !used) return GI_ERR_ARG;
  if (offset + count > c->nlines) return fail(c, GI_ERR_ARG, "line range past the end");
  const SymInfo* sym = sym_info(c->sym_type);
  if (!sym) return fail(c, GI_ERR_STATE, "no symmetry");
  std::vector<gi_line> lines((size_t)count);
  if (count) {
    gi_status st = gi_get_lines(h, offset, count, lines.data());
    if (st != GI_OK) return st;
  }
  const int nmodes = c->params.nmodes;
  const int nclasses = c->trove ? c->trove->nclasses : 0;
  double zpe = c->stats.zpe;
  auto label = [&](int g) -> const char* {
    return (g >= 0 && g < (int)sym->labels.size()) ? sym->labels[g] : "?";
  };
  auto describe = [&](const Level& L, gi_trove_level& out) {
    std::memset(&out, 0, sizeof(out));
    bool have = false;
    if (c->trove) {
      auto it = c->trove->levels.find({L.J, L.gamma});
      if (it != c->trove->levels.end() && L.rec < (int)it->second.size()) {
        out = it->second[L.rec];
        have = true;
      }
    }
    if (!have) {
      auto bit = c->blocks.find({L.J, L.gamma});
      out.ilevel = L.rec;
      out.krot = L.krot;
      out.taurot = L.taurot;
      for (int q = 0; q <= nclasses && q < GI_TROVE_MAXQ; q++) out.cgamma[q] = L.gamma;
      if (bit != c->blocks.end())
        for (int q = 0; q <= nmodes; q++)
          out.quanta[q] = out.normal[q] = bit->second->quanta[(size_t)L.rec * (nmodes + 1) + q];
    }
  };
  std::string s;
  s.reserve((size_t)count * 256);
  for (const gi_line& ln : lines) {
    if (ln.level_i < 0 || ln.level_f < 0 || ln.level_i >= (int)c->levels.size() ||
        ln.level_f >= (int)c->levels.size())
      return fail(c, GI_ERR_STATE, "gi_format_lines: lines carry no level-table ids");
    const Level& LI = c->levels[ln.level_i];
    const Level& LF = c->levels[ln.level_f];
    gi_trove_level dI, dF;
    describe(LI, dI);
    describe(LF, dF);
    gi_line_text f;
    std::memset(&f, 0, sizeof(f));
    f.jF = LF.J;
    f.jI = LI.J;
    f.krotF = dF.krot;
    f.krotI = dI.krot;
    f.ilevelF = dF.ilevel;
    f.ilevelI = dI.ilevel;
    f.nclasses = std::min(nclasses, GI_TROVE_MAXQ - 1);
    f.nmodes = std::min(nmodes, GI_TROVE_MAXQ - 1);
    f.ndegF = ln.ndeg_f;
    f.ndegI = ln.ndeg_i;
    f.symF = label(LF.gamma);
    f.symI = label(LI.gamma);
    for (int q = 0; q <= f.nclasses; q++) {
      f.cgF[q] = label(dF.cgamma[q]);
      f.cgI[q] = label(dI.cgamma[q]);
    }
    for (int q = 0; q <= f.nmodes; q++) {
      f.quantaF[q] = dF.quanta[q];
      f.quantaI[q] = dI.quanta[q];
      f.normalF[q] = dF.normal[q];
      f.normalI[q] = dI.normal[q];
    }
    f.eF = LF.energy - zpe;
    f.eI = LI.energy - zpe;
    f.nu = ln.nu;
    f.S = ln.S;
    f.A = ln.A;
    f.I = ln.I;
    for (int q = 0; q < 4; q++) f.t[q] = ln.t[q];
    format_line_text(f, s);
  }
  *used = s.size();
  if (buf && cap) {
    const size_t n = std::min(cap - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
    if (s.size() >= cap) return fail(c, GI_ERR_ARG, "gi_format_lines: buffer holds %zu of %zu bytes", cap, s.size() + 1);
  }
  return GI_OK;
}

}  // extern "C"
