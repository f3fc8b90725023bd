// The reference's binary snapshot layout for one DM-NRG shell.
//
// CNRGarray::SaveBin (NRGarrayClass.cpp:780-868) writes, in order: Nshell,
// NQNumbers, then for QNumbers, dEn, dEigVec, cEigVec, BlockBegEnd, iDegen,
// Kept a count followed by the elements (int 4 bytes, double 8, complex 16,
// bool 1), then totalS (bool) and Sqnumbers.  CNRGbasisarray::SaveBin
// (:1947-2003) appends iType, StCameFrom, BlockBegEndBC, BlockBegEndEigVec,
// NQNumbers_stcf and StCameFromQNumbers; CNRGmatrix::SaveBin
// (NRGmatrixClass.cpp:957-1015) appends MatEl, MatElCplx, MatBlockMap,
// MatBlockBegEnd, NeedOld, UpperTriangular, IsComplex (bools) and
// WignerEckartL.  What NRG_main leaves in each field for a saved shell with
// UpdateBefCut = 1 (NRG_main.cpp:334-371): Abasis_N as BuildBasis made it
// (no Kept, no eigenvectors); Acut_N the uncut eigen-array (all eigenvectors,
// Kept flags, BlockBegEndBC = BlockBegEnd, StCameFrom = identity); Mat0_N
// (c_d, NeedOld, WignerEckartL 0.5) synced with Acut_N (QNumbers,
// BlockBegEnd, Kept; no dEn).
#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iomanip>
#include <iterator>
#include <string>
#include <vector>

#include "../../include/twochnrg_gb300.h"
#include "nrg_model.h"

namespace {

struct Out {
  std::ofstream f;
  explicit Out(const std::string& path) : f(path, std::ios::out | std::ios::binary | std::ios::trunc) {}
  void i32(int32_t v) { f.write(reinterpret_cast<const char*>(&v), 4); }
  void f64(double v) { f.write(reinterpret_cast<const char*>(&v), 8); }
  void b8(bool v) { const unsigned char c = v ? 1 : 0; f.write(reinterpret_cast<const char*>(&c), 1); }
  void dvec(const double* p, int64_t n) {
    i32((int32_t)n);
    if (n > 0) f.write(reinterpret_cast<const char*>(p), 8 * n);
  }
  void ivec(const int* p, int64_t n) {
    i32((int32_t)n);
    for (int64_t k = 0; k < n; ++k) i32(p[k]);
  }
  void bvec(const unsigned char* p, int64_t n) {
    i32((int32_t)n);
    for (int64_t k = 0; k < n; ++k) b8(p[k] != 0);
  }
};

int nstates_of(const nrg_blocks& b) { return b.nblocks ? b.block_beg_end[2 * b.nblocks - 1] + 1 : 0; }

// The CNRGarray part.
void write_array(Out& o, int nshell, const nrg_blocks& b, const double* en, int64_t nen, const double* evec,
                 int64_t nevec, const unsigned char* kept, int64_t nkept) {
  const int sq = 1;  // position of total S among the quantum numbers (|Q S> models)
  o.i32(nshell);
  o.i32(b.nqn);
  o.dvec(b.qnumbers, (int64_t)b.nblocks * b.nqn);
  o.dvec(en, nen);
  o.dvec(evec, nevec);
  o.i32(0);                                   // cEigVec
  o.ivec(b.block_beg_end, 2 * (int64_t)b.nblocks);
  o.i32(0);                                   // iDegen
  o.bvec(kept, nkept);
  o.b8(true);                                 // totalS
  o.ivec(&sq, 1);                             // Sqnumbers
}

std::string path_of(const char* dir, const char* what, const char* name, int n) {
  return std::string(dir) + "/" + what + "_" + name + "_N" + std::to_string(n) + ".bin";
}

// Reader of the same layout (the inverse of Out): every count is checked
// against the bytes left, so a truncated or foreign file fails cleanly.
struct In {
  std::vector<char> b;
  size_t pos = 0;
  bool ok = true;
  bool need(size_t k) { if (!ok || pos + k > b.size()) ok = false; return ok; }
  int32_t i32() { int32_t v = 0; if (need(4)) { std::memcpy(&v, b.data() + pos, 4); pos += 4; } return v; }
  double f64() { double v = 0; if (need(8)) { std::memcpy(&v, b.data() + pos, 8); pos += 8; } return v; }
  bool b8() { bool v = false; if (need(1)) { v = b[pos] != 0; pos += 1; } return v; }
  int32_t count(size_t elem) {
    const int32_t n = i32();
    if (n < 0 || !need((size_t)n * elem)) { ok = false; return 0; }
    return n;
  }
  void dvec(std::vector<double>& v) {
    const int32_t n = count(8);
    v.resize(n);
    if (n) { std::memcpy(v.data(), b.data() + pos, 8 * (size_t)n); pos += 8 * (size_t)n; }
  }
  void ivec(std::vector<int>& v) {
    const int32_t n = count(4);
    v.resize(n);
    for (int32_t k = 0; k < n; ++k) v[k] = i32();
  }
  void bvec(std::vector<unsigned char>& v) {
    const int32_t n = count(1);
    v.resize(n);
    for (int32_t k = 0; k < n; ++k) v[k] = b8() ? 1 : 0;
  }
  void skip(size_t elem) { const int32_t n = count(elem); pos += (size_t)n * elem; }
};

}  // namespace

namespace nrg {

// CNRGarray::ReadBin / CNRGbasisarray::ReadBin / CNRGmatrix::ReadBin
// (NRGarrayClass.cpp:886-958, 2005-2078; NRGmatrixClass.cpp:1016-1082):
// the fields in SaveBin's order; complex parts and the fields NRG_main
// leaves empty are skipped.  kind: 0 CNRGarray, 1 CNRGbasisarray, 2 CNRGmatrix.
bool read_bin_file(const std::string& path, int kind, BinShellFile& f, std::string& err) {
  std::ifstream is(path, std::ios::in | std::ios::binary);
  if (!is) { err = "cannot open " + path; return false; }
  In in;
  in.b.assign(std::istreambuf_iterator<char>(is), std::istreambuf_iterator<char>());
  f.nshell = in.i32();
  f.nqn = in.i32();
  in.dvec(f.qn);
  in.dvec(f.en);
  in.dvec(f.evec);
  in.skip(16);              // cEigVec
  in.ivec(f.bbe);
  in.skip(4);               // iDegen
  in.bvec(f.kept);
  f.totalS = in.b8();
  in.ivec(f.sqnumbers);
  if (kind == 1) {
    in.ivec(f.itype);
    in.ivec(f.stcf);
    in.ivec(f.bbe_bc);
    in.ivec(f.bbe_eig);
    in.i32();               // NQNumbers_stcf
    in.skip(8);             // StCameFromQNumbers
  } else if (kind == 2) {
    in.dvec(f.mat_el);
    in.skip(16);            // MatElCplx
    in.ivec(f.map);
    in.ivec(f.mbe);
    in.b8(); in.b8(); in.b8();  // NeedOld, UpperTriangular, IsComplex
    in.f64();               // WignerEckartL
  }
  if (!in.ok || in.pos != in.b.size()) { err = "malformed or truncated snapshot " + path; return false; }
  if (f.nqn <= 0 || f.qn.size() % (size_t)f.nqn != 0 || f.bbe.size() != 2 * (f.qn.size() / f.nqn)) {
    err = "inconsistent block structure in " + path;
    return false;
  }
  return true;
}

std::string bin_path(const char* dir, const char* what, const char* name, int n) { return path_of(dir, what, name, n); }

}  // namespace nrg

extern "C" {

nrg_status nrg_write_dm_shell(const char* dir, const char* name, const nrg_dm_shell* s) {
  if (!dir || !name || !s) return NRG_ERR_ARG;
  const nrg_blocks& bb = s->basis.blocks;
  const nrg_blocks& eb = s->blocks;
  if (bb.nqn != 2 || eb.nqn != 2 || !s->en || !s->kept || !s->eigvec) return NRG_ERR_ARG;
  const int nb_states = nstates_of(bb), ne = nstates_of(eb);
  std::vector<int> bc(2 * eb.nblocks), beig(2 * eb.nblocks), ident(ne);
  int64_t nev = 0;
  for (int b = 0; b < eb.nblocks; ++b) {
    const int n = eb.block_beg_end[2 * b + 1] - eb.block_beg_end[2 * b] + 1;
    bc[2 * b] = eb.block_beg_end[2 * b];
    bc[2 * b + 1] = eb.block_beg_end[2 * b + 1];
    beig[2 * b] = (int)nev;
    beig[2 * b + 1] = (int)(nev + (int64_t)n * n - 1);
    nev += (int64_t)n * n;
  }
  for (int i = 0; i < ne; ++i) ident[i] = i;
  {  // Abasis_N
    Out o(path_of(dir, "Abasis", name, s->nshell));
    if (!o.f) return NRG_ERR_ARG;
    write_array(o, s->nshell, bb, s->basis.en, nb_states, nullptr, 0, nullptr, 0);
    o.ivec(s->basis.itype, nb_states);
    o.ivec(s->basis.st_came_from, nb_states);
    o.i32(0);  // BlockBegEndBC
    o.i32(0);  // BlockBegEndEigVec
    o.i32(0);  // NQNumbers_stcf
    o.i32(0);  // StCameFromQNumbers
    if (!o.f.good()) return NRG_ERR_ARG;
  }
  {  // Acut_N
    Out o(path_of(dir, "Acut", name, s->nshell));
    if (!o.f) return NRG_ERR_ARG;
    write_array(o, s->nshell, eb, s->en, ne, s->eigvec, nev, s->kept, ne);
    o.i32(0);  // iType
    o.ivec(ident.data(), ne);
    o.ivec(bc.data(), (int64_t)bc.size());
    o.ivec(beig.data(), (int64_t)beig.size());
    o.i32(0);
    o.i32(0);
    if (!o.f.good()) return NRG_ERR_ARG;
  }
  {  // Mat0_N (c_d)
    Out o(path_of(dir, "Mat0", name, s->nshell));
    if (!o.f) return NRG_ERR_ARG;
    write_array(o, s->nshell, eb, nullptr, 0, nullptr, 0, s->kept, ne);
    const nrg_matrix& m = s->cd;
    int64_t nel = 0;
    for (int k = 0; k < m.nmatblocks; ++k) nel = std::max<int64_t>(nel, (int64_t)m.mat_block_beg_end[2 * k + 1] + 1);
    o.dvec(m.mat_el, nel);
    o.i32(0);  // MatElCplx
    o.ivec(m.mat_block_map, 2 * (int64_t)m.nmatblocks);
    o.ivec(m.mat_block_beg_end, 2 * (int64_t)m.nmatblocks);
    o.b8(true);   // NeedOld
    o.b8(false);  // UpperTriangular
    o.b8(false);  // IsComplex
    o.f64(0.5);   // WignerEckartL
    if (!o.f.good()) return NRG_ERR_ARG;
  }
  return NRG_OK;
}

nrg_status nrg_write_code_pars(const char* dir, double lambda, int nsites, const char* name) {
  if (!dir || !name) return NRG_ERR_ARG;
  std::ofstream f(std::string(dir) + "/ThisCodePars.dat");
  if (!f) return NRG_ERR_ARG;
  // Lambda, Nsites0, Nsitesmax, NopsSaved, SaveArraysFileName, SymNo, ModelNo, BandNo, z_twist
  // (Lambda at full precision: the reader parses it with operator>>)
  f << std::setprecision(17) << lambda << "\n0\n" << nsites << "\n1\n" << name << "\n0\n0\n0\n1\n";
  return f.good() ? NRG_OK : NRG_ERR_ARG;
}

}  // extern "C"
