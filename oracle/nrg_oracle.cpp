// CPU oracle: a plain C++ restatement of the TwoChNRG iterative
// diagonalization (the NRG_main sweep) used ONLY as the checker by tests/,
// __graft_entry__.smoke() and bench.py's CPU baseline.  It is test
// infrastructure, never part of the product path.
//
// Every routine follows the reference function it cites (paths relative to
// the TwoChNRG source tree).  The restatement keeps the reference's data
// model (block-concatenated state vectors, BlockBegEnd pairs, row-wise
// per-block eigenvectors, MatBlockMap/MatBlockBegEnd/MatEl operators), its
// element-by-element Hamiltonian and operator rules and its LAPACK dspev /
// CBLAS dgemm calls, so its arithmetic is that of the reference.  LAPACK and
// BLAS come from the OpenBLAS bundled with scipy, loaded at run time.
//
// Parity pin: the outputs of this file are compared against (a) the
// reference's own golden log Runs/run1/output_NRG_test.txt and (b) full-
// precision fixtures produced by the unmodified reference through
// oracle/ref_harness.cpp (tests/golden/).
#include "nrg_oracle.h"

#include <dlfcn.h>

#include <algorithm>
#include <array>
#include <chrono>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <string>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ---------------------------------------------------------------- LAPACK/BLAS
typedef void (*dspev_t)(const char*, const char*, const int*, double*, double*, double*,
                        const int*, double*, int*, size_t, size_t);
typedef void (*dgemm_t)(int, int, int, int, int, int, double, const double*, int, const double*,
                        int, double, double*, int);
typedef void (*setthreads_t)(int);
dspev_t g_dspev = nullptr;
dgemm_t g_dgemm = nullptr;
setthreads_t g_setthreads = nullptr;
std::string g_err;

const int kRowMajor = 101, kNoTrans = 111, kTrans = 112;

// ---------------------------------------------------------------- helpers
// dEqual.cpp:6 — absolute 1e-20 comparison used for quantum numbers.
inline bool dEq(double a, double b) { return std::fabs(a - b) < 1.e-20; }
// dEqual.cpp:17 — A<B or |A-B|<1e-20.
inline bool dLEq(double a, double b) { return (a < b) || (std::fabs(a - b) < 1.e-20); }

// gsl_sf_fact(n): n! rounded once to double (exact integer product in 128 bits).
double fact(int n) {
  if (n < 0) return 0.0;
  unsigned __int128 p = 1;
  for (int k = 2; k <= n; ++k) p *= (unsigned)k;
  return (double)p;
}

// CGordan.cpp:34-120 — Clebsch-Gordan <J1 M1; J2 M2 | J M> (Landau-Lifshitz form).
double cgordan(double J1, double M1, double J2, double M2, double J, double M) {
  if ((J1 < 0.0) || (J2 < 0.0) || (J < 0.0)) return 0.0;
  if ((std::fabs(M1) > J1) || (std::fabs(M2) > J2) || (std::fabs(M) > J)) return 0.0;
  if (std::fabs(M - (M1 + M2)) > 1.0e-10) return 0.0;
  if ((J > (J1 + J2)) || (J < std::fabs(J1 - J2))) return 0.0;
  double a0 = fact((int)(J1 + J2 - J)), a1 = fact((int)(J1 - J2 + J)), a2 = fact((int)(-J1 + J2 + J));
  double a3 = 2 * J + 1, a4 = fact((int)(J1 + J2 + J + 1));
  double a5 = a0 * a1 * a2 * a3 / a4;
  double rho = a5 > 0.0 ? std::sqrt(a5) : 0.0;
  double s0 = fact((int)(J + M)), s1 = fact((int)(J - M)), s2 = fact((int)(J1 + M1));
  double s3 = fact((int)(J1 - M1)), s4 = fact((int)(J2 + M2)), s5 = fact((int)(J2 - M2));
  double s6 = s0 * s1 * s2 * s3 * s4 * s5;
  double sigma = s6 > 0.0 ? std::sqrt(s6) : 0.0;
  int b1[] = {(int)(J1 - M1), (int)(J2 + M2), (int)(J1 + J2 - J)};
  int rmax = *std::min_element(b1, b1 + 3);
  int b2[] = {-(int)(J - J2 + M1), -(int)(J - J1 - M2), 0};
  int rmin = *std::max_element(b2, b2 + 3);
  double tau = 0.0;
  for (int r = rmin; r <= rmax; r++) {
    double t0 = fact((int)(J1 - M1) - r), t1 = fact((int)(J2 + M2) - r), t2 = fact((int)(J - J2 + M1) + r);
    double t3 = fact((int)(J - J1 - M2) + r), t4 = fact((int)(J1 + J2 - J) - r), t5 = fact(r);
    double t6 = 1.0 / (t0 * t1 * t2 * t3 * t4 * t5);
    tau += std::pow(-1.0, r) * t6;
  }
  return rho * sigma * tau;
}

// CGordan.cpp:13 — triangle inequality with a 1e-10 tolerance.
bool triang(double J1, double J2, double J) {
  return !((J - (J1 + J2) > 1.0e-10) || (J - std::fabs(J1 - J2) < -1.0e-10));
}

// Memoised CG: the reference calls CGordan ~1e7 times per sweep; the value is
// a pure function of its six arguments, so caching it changes no result.
struct CGCache {
  std::map<std::array<double, 6>, double> m;
  double operator()(double a, double b, double c, double d, double e, double f) {
    std::array<double, 6> k{a, b, c, d, e, f};
    auto it = m.find(k);
    if (it != m.end()) return it->second;
    double v = cgordan(a, b, c, d, e, f);
    m.emplace(k, v);
    return v;
  }
};

// ---------------------------------------------------------------- containers
// CNRGarray (include/NRGclasses.hpp:47-200).
struct Arr {
  int nshell = 0, nqn = 0;
  std::vector<double> qn;
  std::vector<int> bbe;         // BlockBegEnd pairs
  std::vector<double> en;       // dEn
  std::vector<double> evec;     // dEigVec, block-concatenated, row = eigenvector
  std::vector<char> kept;       // Kept
  bool totalS = false;
  std::vector<int> sqn;         // Sqnumbers
  int nblocks() const { return nqn ? (int)qn.size() / nqn : 0; }
  int beg(int b) const { return b < 0 ? 0 : bbe[2 * b]; }
  int end(int b) const { return b < 0 ? 0 : bbe[2 * b + 1]; }
  int bsize(int b) const { return bbe[2 * b + 1] - bbe[2 * b] + 1; }
  int nstates() const { return bbe.empty() ? 0 : bbe.back() - bbe.front() + 1; }
  double q(int b, int k) const { return qn.empty() ? 0.0 : qn[(size_t)b * nqn + k]; }
  // GetBlockFromSt (NRGarrayClass.cpp:374): first block whose end >= ist.
  int block_of(int ist, int& pos) const {
    int lo = 0, hi = nblocks() - 1;
    while (lo < hi) {
      int mid = (lo + hi) / 2;
      if (ist > bbe[2 * mid + 1]) lo = mid + 1; else hi = mid;
    }
    pos = ist - bbe[2 * lo];
    return lo;
  }
  // GetBlockFromQNumbers (NRGarrayClass.cpp:514): first block whose QNs all
  // match within 1e-20, -1 if none.
  int block_of_qn(const double* q) const {
    for (int b = 0; b < nblocks(); ++b) {
      bool ok = true;
      for (int k = 0; k < nqn && ok; ++k) ok = dEq(qn[(size_t)b * nqn + k], q[k]);
      if (ok) return b;
    }
    return -1;
  }
};

// CNRGbasisarray (NRGclasses.hpp:215-349).
struct Basis : Arr {
  std::vector<int> itype, stcf, bbe_bc, bbe_eig;
  int bsize_bc(int b) const { return bbe_bc[2 * b + 1] - bbe_bc[2 * b] + 1; }
};

// CNRGmatrix (NRGclasses.hpp:365-759) for real, non-packed operators.
struct Mat {
  Arr blk;                         // the synced block structure it acts on
  std::vector<int> map, mbe;
  std::vector<double> el;
  std::map<std::pair<int, int>, int> index;  // FindMatBlock (NRGmatrixClass.cpp:33)
  bool need_old = false, calc_avg = false;
  std::string name;
  int rule = 0;  // operator rule id (see OpRule)
  void clear_data() { map.clear(); mbe.clear(); el.clear(); index.clear(); }
  void push_block(int i, int j, const double* v, int n) {
    index.emplace(std::make_pair(i, j), (int)map.size() / 2);
    map.push_back(i); map.push_back(j);
    int b = (int)el.size();
    mbe.push_back(b); mbe.push_back(b + n - 1);
    el.insert(el.end(), v, v + n);
  }
  // GetMatEl (NRGmatrixClass.cpp:174) -> GetBlockMatEl (:131).
  double get(int ist, int jst) const {
    int pi, pj;
    int bi = blk.block_of(ist, pi), bj = blk.block_of(jst, pj);
    auto it = index.find(std::make_pair(bi, bj));
    if (it == index.end() || pi < 0 || pj < 0) return 0.0;
    int n2 = blk.bsize(bj);
    return el[(size_t)mbe[2 * it->second] + (size_t)pi * n2 + pj];
  }
};

// ---------------------------------------------------------------- site tables
// OneCh_fd_table (OpTables.cpp:8-33): <type_i| f^dagger_sigma |type_j>.
double onech_fd(int sigma, int ti, int tj) {
  if (sigma == 1) { if (ti == 1 && tj == 0) return 1.0; if (ti == 3 && tj == 2) return 1.0; return 0.0; }
  if (sigma == -1) { if (ti == 2 && tj == 0) return 1.0; if (ti == 3 && tj == 1) return -1.0; return 0.0; }
  return 0.0;
}

// OneChS_fd_table (OpTables.cpp:419-443) in the basis |0>, |up dn>, |up>, |dn>
// of the superconducting-lead site, and OneChS_fdupfddn_table (:447-462).
double onechS_fd(int sigma, int ti, int tj) {
  if (sigma == 1) { if (ti == 2 && tj == 0) return 1.0; if (ti == 1 && tj == 3) return 1.0; return 0.0; }
  if (sigma == -1) { if (ti == 3 && tj == 0) return 1.0; if (ti == 1 && tj == 2) return -1.0; return 0.0; }
  return 0.0;
}
double onechS_pair(int ti, int tj) { return (ti == 1 && tj == 0) ? 1.0 : 0.0; }

// TwoChQS_fd_table (TwoChQS_OpTables.cpp:20-130) in the 16-state site basis
// of TwoChQS_SetSingleSite.  The table entries are the reference's.
double twoch_fd(int ch, int sigma, int ti, int tj) {
  if (ti < 0 || tj < 0 || ti > 15 || tj > 15) return 0.0;
  double M[16][16] = {{0.0}};
  const double r = 1.0 / std::sqrt(2.0), mr = -1.0 / std::sqrt(2.0);
  if (ch == 1 && sigma == 1) {
    M[2][0] = 1; M[10][1] = 1; M[9][3] = r; M[11][6] = 1; M[5][3] = r;
    M[7][4] = 1; M[12][9] = r; M[12][5] = mr; M[14][8] = 1; M[15][13] = 1;
  } else if (ch == 1 && sigma == -1) {
    M[4][0] = 1; M[9][1] = r; M[5][1] = mr; M[8][3] = 1; M[13][6] = 1;
    M[7][2] = -1; M[12][10] = -1; M[14][9] = mr; M[14][5] = mr; M[15][11] = -1;
  } else if (ch == 2 && sigma == 1) {
    M[1][0] = 1; M[6][3] = 1; M[10][2] = -1; M[11][9] = mr; M[11][5] = mr;
    M[9][4] = mr; M[5][4] = r; M[13][8] = -1; M[12][7] = 1; M[15][14] = 1;
  } else if (ch == 2 && sigma == -1) {
    M[3][0] = 1; M[6][1] = -1; M[9][2] = mr; M[11][10] = 1; M[5][2] = mr;
    M[8][4] = -1; M[13][9] = r; M[13][5] = mr; M[14][7] = 1; M[15][12] = -1;
  } else {
    return 0.0;
  }
  return M[ti][tj];
}

// TwoChQS_SpSm_table (TwoChQS_OpTables.cpp:140-185): 1 on the diagonal and on
// the pairs connected by S+/S- within a channel, else 0.
double twoch_spsm(int ti, int tj) {
  if (ti == tj) return 1.0;
  static const int pairs[][2] = {{1, 3}, {2, 4}, {11, 13}, {12, 14}, {8, 9}, {9, 10}, {8, 10}};
  for (auto& p : pairs)
    if ((p[0] == ti && p[1] == tj) || (p[1] == ti && p[0] == tj)) return 1.0;
  return 0.0;
}

void add_site_block(Basis& s, std::initializer_list<double> q, int b, int e) {
  for (double v : q) s.qn.push_back(v);
  s.bbe.push_back(b); s.bbe.push_back(e);
}

// OneChQS_SetSingleSite (OneChQS_SetSingleSite.cpp:5-44).
Basis site_1chQS() {
  Basis s; s.nqn = 3; s.totalS = true; s.sqn = {1};
  add_site_block(s, {-1, 0, 0}, 0, 0); add_site_block(s, {0, 0.5, 0.5}, 1, 1);
  add_site_block(s, {0, 0.5, -0.5}, 2, 2); add_site_block(s, {1, 0, 0}, 3, 3);
  for (int i = 0; i < 4; ++i) s.itype.push_back(i);
  return s;
}
// OneChQSz_SetSingleSite (Main/Main_SetSingleSite.cpp:347-380).
Basis site_1chQSz() {
  Basis s; s.nqn = 2; s.totalS = false;
  add_site_block(s, {-1, 0}, 0, 0); add_site_block(s, {0, 0.5}, 1, 1);
  add_site_block(s, {0, -0.5}, 2, 2); add_site_block(s, {1, 0}, 3, 3);
  for (int i = 0; i < 4; ++i) s.itype.push_back(i);
  return s;
}
// CNRGCodeHandler::SetSingleSite for SymNo 3 (NRGcodehandlerClass.cpp:484-503).
// CNRGCodeHandler::SetSingleSite for SymNo 7 (NRGcodehandlerClass.cpp:536-560):
// (S,Sz) blocks |0>,|up dn> | |up> | |dn>.
Basis site_1chS() {
  Basis s; s.nqn = 2; s.totalS = true; s.sqn = {0};
  add_site_block(s, {0, 0}, 0, 1); add_site_block(s, {0.5, 0.5}, 2, 2); add_site_block(s, {0.5, -0.5}, 3, 3);
  for (int i = 0; i < 4; ++i) s.itype.push_back(i);
  return s;
}
// CNRGCodeHandler::SetSingleSite for SymNo 8 (NRGcodehandlerClass.cpp:564-584):
// Sz blocks |0>,|up dn> | |up> | |dn>.
Basis site_1chSz() {
  Basis s; s.nqn = 1; s.totalS = false;
  add_site_block(s, {0}, 0, 1); add_site_block(s, {0.5}, 2, 2); add_site_block(s, {-0.5}, 3, 3);
  for (int i = 0; i < 4; ++i) s.itype.push_back(i);
  return s;
}
Basis site_1chQ() {
  Basis s; s.nqn = 1; s.totalS = false;
  add_site_block(s, {-1}, 0, 0); add_site_block(s, {0}, 1, 2); add_site_block(s, {1}, 3, 3);
  for (int i = 0; i < 4; ++i) s.itype.push_back(i);
  return s;
}
// TwoChQS_SetSingleSite (TwoChQS_SetSingleSite.cpp:5-124): 16 states in 10 blocks.
Basis site_2chQS() {
  Basis s; s.nqn = 3; s.totalS = true; s.sqn = {1};
  add_site_block(s, {-2, 0, 0}, 0, 0);
  add_site_block(s, {-1, 0.5, 0.5}, 1, 2);
  add_site_block(s, {-1, 0.5, -0.5}, 3, 4);
  add_site_block(s, {0, 0, 0}, 5, 7);
  add_site_block(s, {0, 1, -1}, 8, 8);
  add_site_block(s, {0, 1, 0}, 9, 9);
  add_site_block(s, {0, 1, 1}, 10, 10);
  add_site_block(s, {1, 0.5, 0.5}, 11, 12);
  add_site_block(s, {1, 0.5, -0.5}, 13, 14);
  add_site_block(s, {2, 0, 0}, 15, 15);
  for (int i = 0; i < 16; ++i) s.itype.push_back(i);
  return s;
}

// ---------------------------------------------------------------- rules
enum OpRule { R_F_QS = 1, R_FUP_QSZ, R_FDN_QSZ, R_F1_2CH, R_F2_2CH, R_IMPONLY, R_CD_QS, R_F_S, R_FUP_SZ, R_FDN_SZ,
              R_CD_2CH };
enum Check { C_DIAG = 1, C_QS_CD, C_Q_CD, C_2CH_CD, C_S_CD, C_SZ_UP, C_SZ_DN };

struct Model {
  int kind;          // ORACLE_MODEL_*
  Basis site;
  std::vector<int> common{2, 0, 1, 0, 1}, totS;
  int nchan = 1;
  std::vector<int> op_rule, op_check;  // per operator
};

// CheckForMatEl rules: Diag_check OpMatRules.cpp:12, OneChQS_cd_check :106,
// OneChQ_cd_check :92, TwoChQS_cd_check TwoChQS_OpMatRules.cpp:16.
bool check(int c, const Arr& a, int i, int j) {
  switch (c) {
    case C_DIAG: return i == j;
    case C_QS_CD: return dEq(a.q(j, 0), a.q(i, 0) + 1.0) &&
                         (dEq(a.q(j, 1), a.q(i, 1) + 0.5) || dEq(a.q(j, 1), a.q(i, 1) - 0.5));
    case C_Q_CD: return dEq(a.q(j, 0), a.q(i, 0) + 1.0);
    case C_2CH_CD: return dEq(a.q(j, 0), a.q(i, 0) + 1.0) &&
                          (dEq(a.q(j, 1), a.q(i, 1) + 0.5) || dEq(a.q(j, 1), a.q(i, 1) - 0.5));
    case C_S_CD: return dEq(a.q(j, 0), a.q(i, 0) + 0.5) || dEq(a.q(j, 0), a.q(i, 0) - 0.5);  // OneChS_cd_check :172
    case C_SZ_UP: return dEq(a.q(j, 0), a.q(i, 0) + 0.5);  // OneChSz_cdup_check :188
    case C_SZ_DN: return dEq(a.q(j, 0), a.q(i, 0) - 0.5);  // OneChSz_cddn_check :199
  }
  return false;
}

struct Ctx {
  Model m;
  CGCache cg;
};

double qn_from_st(const Arr& a, int ist, int k) { int p; int b = a.block_of(ist, p); return a.q(b, k); }

// OneChQS_HN_MatEl (OpMatRules.cpp:1410-1535).
double hn_1chQS(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
                int ist, int jst) {
  const Basis& ss = c.m.site;
  double Lambda = P[0], chi_N = P[1], eN = P[2];
  double Qi = qn_from_st(ab, ist, 0), Si = qn_from_st(ab, ist, 1);
  double Qj = qn_from_st(ab, jst, 0), Sj = qn_from_st(ab, jst, 1);
  if (!dEq(Qi, Qj) || !dEq(Si, Sj)) return 0.0;
  if (ist == jst) {
    double v = std::sqrt(Lambda) * ab.en[ist];
    double Qt = qn_from_st(ss, ab.itype[ist], 0);
    return v + eN * (Qt + 1.0);
  }
  int ti = ab.itype[ist], tj = ab.itype[jst];
  double Old = M[0].get(ab.stcf[ist], ab.stcf[jst]);
  int typep = ti, type = tj;
  if (dEq(Old, 0.0)) { Old = M[0].get(ab.stcf[jst], ab.stcf[ist]); typep = tj; type = ti; }
  double Qtp = ss.q(typep, 0), Stp = ss.q(typep, 1), Sztp = ss.q(typep, 2);
  double Qt = ss.q(type, 0), St = ss.q(type, 1), Szt = ss.q(type, 2);
  double Scfp = Si - Sztp, Scf = Si - Szt;
  double FermiSign = dEq(Qt, 0.0) ? -1.0 : 1.0;
  double Coef = 0.0;
  double sqp[3] = {Qtp, Stp, Sztp}, sq[3] = {Qt, St, Szt};
  for (double Sz = -St; Sz <= St; Sz += 1.0) {
    sq[2] = Sz;
    int sst = ss.block_of_qn(sq);
    for (int sigma = -1; sigma <= 1; sigma += 2) {
      double dS = 0.5 * (double)sigma;
      double Szcf = Si - Sz, Szcfp = Szcf - dS, Szp = Sz + dS;
      sqp[2] = Sz + dS;
      int sstp = ss.block_of_qn(sqp);
      double a0 = c.cg(Scf, Szcf, St, Sz, Si, Si);
      double a1 = c.cg(Scfp, Szcfp, Stp, Szp, Si, Si);
      double a2 = c.cg(Scfp, Szcfp, 0.5, dS, Scf, Szcf);
      double a3 = onech_fd(sigma, sstp, sst);
      Coef += a0 * a1 * a2 * a3;
    }
  }
  return chi_N * Old * Coef * FermiSign;
}

// OneChQSz_HN_MatEl (OpMatRules.cpp:431-537).
double hn_1chQSz(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
                 int ist, int jst) {
  const Basis& ss = c.m.site;
  double Lambda = P[0], chi_N = P[1], eN = P[2];
  double Qi = qn_from_st(ab, ist, 0), Szi = qn_from_st(ab, ist, 1);
  double Qj = qn_from_st(ab, jst, 0), Szj = qn_from_st(ab, jst, 1);
  if (!dEq(Qi, Qj) || !dEq(Szi, Szj)) return 0.0;
  if (ist == jst) {
    double v = std::sqrt(Lambda) * ab.en[ist];
    double Qt = qn_from_st(ss, ab.itype[ist], 0);
    return v + eN * (Qt + 1.0);
  }
  int ti = ab.itype[ist], tj = ab.itype[jst];
  double v = 0.0;
  int imat = 0;
  for (int isigma = 1; isigma >= -1; isigma -= 2) {
    int typep = ti, type = tj;
    double Old = M[imat].get(ab.stcf[ist], ab.stcf[jst]);
    if (dEq(Old, 0.0)) { Old = M[imat].get(ab.stcf[jst], ab.stcf[ist]); typep = tj; type = ti; }
    double Qt = qn_from_st(ss, type, 0);
    double FermiSign = dEq(Qt, 0.0) ? -1.0 : 1.0;
    v += FermiSign * Old * onech_fd(isigma, typep, type);
    imat++;
  }
  return v * chi_N;
}

// OneChS_HNsc_MatEl (OpMatRules.cpp:1794-2003): superconducting leads, S
// blocks.  P = {Lambda, chi_N, e_N, Delta_N}.  The pairing term acts between
// states from the same old state; the hopping reads the old operator
// backwards when its element vanishes or the site table has no f^dagger
// between the two types.
double hn_1chS(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
               int ist, int jst) {
  const Basis& ss = c.m.site;
  double Lambda = P[0], chi_N = P[1], eN = P[2], Delta = P[3];
  double Si = qn_from_st(ab, ist, 0), Sj = qn_from_st(ab, jst, 0);
  if (!dEq(Si, Sj)) return 0.0;
  double v = 0.0;
  if (ist == jst) {
    const double auxN[4] = {0.0, 2.0, 1.0, 1.0};
    v = std::sqrt(Lambda) * ab.en[ist];
    v += eN * auxN[ab.itype[ist]];
    return v;
  }
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (ab.stcf[ist] == ab.stcf[jst]) {
    v -= Delta * onechS_pair(ti, tj);
    v -= Delta * onechS_pair(tj, ti);
    return v;
  }
  double Old = M[0].get(ab.stcf[ist], ab.stcf[jst]);
  int typep = ti, type = tj;
  if (dEq(Old, 0.0) || (dEq(onechS_fd(1, ti, tj), 0.0) && dEq(onechS_fd(-1, ti, tj), 0.0))) {
    Old = M[0].get(ab.stcf[jst], ab.stcf[ist]);
    typep = tj; type = ti;
  }
  double Stp = qn_from_st(ss, typep, 0), Sztp = qn_from_st(ss, typep, 1);
  double St = qn_from_st(ss, type, 0), Szt0 = qn_from_st(ss, type, 1);
  double Scfp = Si - Sztp, Scf = Si - Szt0;
  double FermiSign = (type == 2 || type == 3) ? -1.0 : 1.0;
  double Coef = 0.0;
  double qp[2] = {Stp, Sztp}, q[2] = {St, Szt0};
  for (double Szt = -St; Szt <= St; Szt += 1.0) {
    q[1] = Szt;
    int sst = type;
    if (type == 2 || type == 3) sst = ss.block_of_qn(q) + 1;
    for (int sigma = -1; sigma <= 1; sigma += 2) {
      double dS = 0.5 * (double)sigma;
      double Szcf = Si - Szt, Szcfp = Szcf - dS, Sztp_ = Szt + dS;
      qp[1] = Sztp_;
      int sstp = ss.block_of_qn(qp) + 1;
      if (dEq(Sztp_, 0.0)) sstp = typep;
      double a0 = c.cg(Scf, Szcf, St, Szt, Si, Si);
      double a1 = c.cg(Scfp, Szcfp, Stp, Sztp_, Si, Si);
      double a2 = c.cg(Scfp, Szcfp, 0.5, dS, Scf, Szcf);
      double a3 = onechS_fd(sigma, sstp, sst);
      Coef += a0 * a1 * a2 * a3;
    }
  }
  v += chi_N * Old * Coef * FermiSign;
  return v;
}

// OneChSz_HNsc_MatEl (OpMatRules.cpp:2098-2205): superconducting leads, Sz
// blocks, f_up and f_dn; per spin the old operator is read backwards when
// its element vanishes or OneChS_fd_table(sigma, t_i, t_j) does.
double hn_1chSz(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
                int ist, int jst) {
  (void)c;
  double Lambda = P[0], chi_N = P[1], eN = P[2], Delta = P[3];
  double Szi = qn_from_st(ab, ist, 0), Szj = qn_from_st(ab, jst, 0);
  if (!dEq(Szi, Szj)) return 0.0;
  double v = 0.0;
  if (ist == jst) {
    const double auxN[4] = {0.0, 2.0, 1.0, 1.0};
    v = std::sqrt(Lambda) * ab.en[ist];
    v += eN * auxN[ab.itype[ist]];
    return v;
  }
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (ab.stcf[ist] == ab.stcf[jst]) {
    v -= Delta * onechS_pair(ti, tj);
    v -= Delta * onechS_pair(tj, ti);
    return v;
  }
  int imat = 0;
  for (int isigma = 1; isigma >= -1; isigma -= 2) {
    double Old = M[imat].get(ab.stcf[ist], ab.stcf[jst]);
    int typep = ti, type = tj;
    if (dEq(Old, 0.0) || dEq(onechS_fd(isigma, ti, tj), 0.0)) {
      Old = M[imat].get(ab.stcf[jst], ab.stcf[ist]);
      typep = tj; type = ti;
    }
    double FermiSign = (type == 2 || type == 3) ? -1.0 : 1.0;
    v += FermiSign * Old * onechS_fd(isigma, typep, type);
    imat++;
  }
  v *= chi_N;
  return v;
}

// OneChQ_HN_MatEl (OpMatRules.cpp:1065-1147): blocks by Q alone, no e_N term.
double hn_1chQ(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
               int ist, int jst) {
  const Basis& ss = c.m.site;
  double Lambda = P[0], chi_N = P[1];
  double Qi = qn_from_st(ab, ist, 0), Qj = qn_from_st(ab, jst, 0);
  if (!dEq(Qi, Qj)) return 0.0;
  if (ist == jst) return std::sqrt(Lambda) * ab.en[ist];
  int ti = ab.itype[ist], tj = ab.itype[jst];
  double v = 0.0;
  int imat = 0;
  for (int isigma = 1; isigma >= -1; isigma -= 2) {
    int typep = ti, type = tj;
    double Old = M[imat].get(ab.stcf[ist], ab.stcf[jst]);
    if (dEq(Old, 0.0)) { Old = M[imat].get(ab.stcf[jst], ab.stcf[ist]); typep = tj; type = ti; }
    double Qt = qn_from_st(ss, type, 0);
    double FermiSign = dEq(Qt, 0.0) ? -1.0 : 1.0;
    v += FermiSign * Old * onech_fd(isigma, typep, type);
    imat++;
  }
  return v * chi_N;
}

// TwoChQS_HN_MatEl (TwoChQS_OpMatRules.cpp:794-986).
double hn_2chQS(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
                int ist, int jst) {
  const Basis& ss = c.m.site;
  double Lambda = P[0], chi[2] = {P[1], P[2]};
  double Qi = qn_from_st(ab, ist, 0), Si = qn_from_st(ab, ist, 1);
  double Qj = qn_from_st(ab, jst, 0), Sj = qn_from_st(ab, jst, 1);
  if (!dEq(Qi, Qj) || !dEq(Si, Sj)) return 0.0;
  if (ist == jst) return std::sqrt(Lambda) * ab.en[ist];
  double v = 0.0;
  int ti = ab.itype[ist], tj = ab.itype[jst];
  int ci = ab.stcf[ist], cj = ab.stcf[jst];
  for (int ich = 1; ich <= 2; ich++) {
    double Old = M[ich - 1].get(ci, cj);
    int typep = ti, type = tj;
    if (dEq(std::fabs(Old), 0.0)) { Old = M[ich - 1].get(cj, ci); typep = tj; type = ti; }
    int pos;
    int bp = ss.block_of(typep, pos), b = ss.block_of(type, pos);
    double Stp = ss.q(bp, 1), Sztp = ss.q(bp, 2);
    double St = ss.q(b, 1), Szt = ss.q(b, 2);
    double Soldp = Si - Sztp, Sold = Si - Szt;
    double FermiSign = (dEq(Szt, 0.5) || dEq(Szt, -0.5)) ? -1.0 : 1.0;
    double sqp[3] = {ss.q(bp, 0), ss.q(bp, 1), ss.q(bp, 2)};
    double sq[3] = {ss.q(b, 0), ss.q(b, 1), ss.q(b, 2)};
    for (int sigma = -1; sigma <= 1; sigma += 2) {
      double dS = 0.5 * (double)sigma;
      double Full = 0.0;
      for (double Szold = Sold; Szold >= -Sold; Szold -= 1.0) {
        double Szoldp = Szold - dS;
        double Sz = Si - Szold, Szp = Sz + dS;
        sqp[2] = Szp; sq[2] = Sz;
        int sbp = ss.block_of_qn(sqp), sb = ss.block_of_qn(sq);
        if (dLEq(std::fabs(Szp), Stp) && dLEq(std::fabs(Szold), Sold) && dLEq(std::fabs(Szoldp), Soldp)) {
          double a0 = c.cg(Sold, Szold, St, Sz, Si, Si);
          double a1 = c.cg(Soldp, Szoldp, Stp, Szp, Si, Si);
          double a2 = c.cg(Soldp, Szoldp, 0.5, dS, Sold, Szold);
          for (int sp = ss.beg(sbp); sp <= ss.end(sbp); sp++)
            for (int s = ss.beg(sb); s <= ss.end(sb); s++) {
              double x0 = twoch_spsm(s, type), x1 = twoch_spsm(sp, typep);
              double a3 = twoch_fd(ich, sigma, sp, s);
              Full += a0 * a1 * a2 * a3 * FermiSign * x0 * x1;
            }
        }
      }
      v += chi[ich - 1] * Old * Full;
    }
  }
  return v;
}

// OneChQS_fN_MatEl (OpMatRules.cpp:1167-1244).
double op_f_QS(Ctx& c, const Basis& ab, int ist, int jst) {
  const Basis& ss = c.m.site;
  double Si = qn_from_st(ab, ist, 1), Sj = qn_from_st(ab, jst, 1);
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (ab.stcf[ist] != ab.stcf[jst]) return 0.0;
  double Qti = ss.q(ti, 0), Sti = ss.q(ti, 1), Szti = ss.q(ti, 2);
  double Qtj = ss.q(tj, 0), Stj = ss.q(tj, 1), Sztj = ss.q(tj, 2);
  double sqi[3] = {Qti, Sti, Szti}, sqj[3] = {Qtj, Stj, Sztj};
  double Scfi = Si - Szti, Scfj = Sj - Sztj;
  double aux0 = 0.0, cg0 = 0.0, cg1 = 0.0;
  double sigma = Sj - Si;
  for (double Sz = -Stj; Sz <= Stj; Sz += 1.0) {
    sqj[2] = Sz;
    int ssj = ss.block_of_qn(sqj);
    sqi[2] = Sz - sigma;
    int ssi = ss.block_of_qn(sqi);
    cg0 = c.cg(Scfi, Si - Sz + sigma, Sti, Sz - sigma, Si, Si);
    cg1 = c.cg(Scfj, Sj - Sz, Stj, Sz, Sj, Sj);
    aux0 += onech_fd((int)(sigma / 0.5), ssj, ssi) * cg0 * cg1;
  }
  double n0 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
  if (!dEq(n0, 0.0)) return aux0 / n0;
  if (!dEq(cg1, 0.0)) return 0.0 / cg1;
  return 0.0;
}

// OneChQ_fN_MatEl (OpMatRules.cpp:1003-1033), sigma = +1 (up) / -1 (dn).
double op_f_QSz(const Basis& ab, int ist, int jst, int isigma) {
  if (ab.stcf[ist] == ab.stcf[jst]) return onech_fd(isigma, ab.itype[jst], ab.itype[ist]);
  return 0.0;
}

// TwoChQS_fN_MatEl (TwoChQS_OpMatRules.cpp:1205-1352).
double op_f_2ch(Ctx& c, const Basis& ab, int ist, int jst, int ich) {
  const Basis& ss = c.m.site;
  double Si = qn_from_st(ab, ist, 1), Sj = qn_from_st(ab, jst, 1);
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (ab.stcf[ist] != ab.stcf[jst]) return 0.0;
  int pos;
  int bi = ss.block_of(ti, pos), bj = ss.block_of(tj, pos);
  double Sti = ss.q(bi, 1), Szti = ss.q(bi, 2), Stj = ss.q(bj, 1), Sztj = ss.q(bj, 2);
  (void)Sti; (void)Stj;
  double sqi[3] = {ss.q(bi, 0), ss.q(bi, 1), ss.q(bi, 2)};
  double sqj[3] = {ss.q(bj, 0), ss.q(bj, 1), ss.q(bj, 2)};
  double Scfi = Si - Szti, Scfj = Sj - Sztj;
  double aux = 0.0, CGnorm = 1.0;
  int sigma = 0;
  double c0 = c.cg(Si, Si, 0.5, -0.5, Sj, Sj), c1 = c.cg(Si, Si, 0.5, 0.5, Sj, Sj);
  if (!dEq(c0, 0.0)) { sigma = -1; CGnorm = c0; }
  else if (!dEq(c1, 0.0)) { sigma = 1; CGnorm = c1; }
  if (sigma == 0) return 0.0;
  for (double Szcfj = Scfj; Szcfj >= -Scfj; Szcfj -= 1.0) {
    double Szi = Si - Szcfj, Szj = Sj - Szcfj;
    sqi[2] = Szi; int bsi = ss.block_of_qn(sqi);
    sqj[2] = Szj; int bsj = ss.block_of_qn(sqj);
    double a0 = c.cg(Scfi, Szcfj, ss.q(bi, 1), Szi, Si, Si);
    double a1 = c.cg(Scfj, Szcfj, ss.q(bj, 1), Szj, Sj, Sj);
    for (int si = ss.beg(bsi); si <= ss.end(bsi); si++)
      for (int sj = ss.beg(bsj); sj <= ss.end(bsj); sj++)
        aux += twoch_fd(ich, sigma, sj, si) * a0 * a1 * twoch_spsm(si, ti) * twoch_spsm(sj, tj);
  }
  return aux / CGnorm;
}

// OneChQS_cd_MatEl (OpMatRules.cpp:1249-1330): the impurity d operator
// between new-basis states (reduced matrix element, SU(2) recoupling of the
// old state with the unchanged site state); multiplied by the old operator by
// UpdateMatrices (NeedOld).  A site state that is not found compares equal to
// another one that is not found (-1 == -1), as in the reference.
double op_cd_QS(Ctx& c, const Basis& ab, int ist, int jst) {
  const Basis& ss = c.m.site;
  double Si = qn_from_st(ab, ist, 1), Sj = qn_from_st(ab, jst, 1);
  int ti = ab.itype[ist], tj = ab.itype[jst];
  double Qti = ss.q(ti, 0), Sti = ss.q(ti, 1), Szti = ss.q(ti, 2);
  double Qtj = ss.q(tj, 0), Stj = ss.q(tj, 1), Sztj = ss.q(tj, 2);
  double sqi[3] = {Qti, Sti, Szti}, sqj[3] = {Qtj, Stj, Sztj};
  double Scfi = Si - Szti, Scfj = Sj - Sztj;
  double f = 0.0;
  double sigma = Sj - Si;
  double a3 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
  if (dEq(a3, 0.0)) {
    sigma = Si - Sj;
    a3 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (dEq(a3, 0.0)) return 0.0;
  }
  for (double Szcfj = -Scfj; Szcfj <= Scfj; Szcfj += 1.0) {
    double Szcfi = Szcfj - sigma;
    double Sztj_ = Sj - Szcfj, Szti_ = Si - Szcfi;
    sqj[2] = Sztj_;
    int sj = ss.block_of_qn(sqj);
    sqi[2] = Szti_;
    int si = ss.block_of_qn(sqi);
    double a0 = c.cg(Scfi, Szcfi, Sti, Szti_, Si, Si);
    double a1 = c.cg(Scfj, Szcfj, Stj, Sztj_, Sj, Sj);
    double a2 = c.cg(Scfi, Szcfi, 0.5, sigma, Scfj, Szcfj);
    double FermiSign = dEq(Qtj, 0.0) ? -1.0 : 1.0;
    if (si == sj) f += a0 * a1 * a2 * FermiSign;
  }
  if (!dEq(a3, 0.0)) f = f / a3; else f = 0.0;
  return f;
}

// The impurity d operator across the 16-state two-channel site.  The
// reference has no such rule (TwoChQS keeps no c_d); this restates
// OneChQS_cd_MatEl's recoupling (above) with the site multiplet unchanged:
// the two types are members of one multiplet (TwoChQS_SpSm_table), the site
// member is the same on both sides, and the Fermi sign is (-1) to the site's
// fermion number Q + 2.
double op_cd_2ch(Ctx& c, const Basis& ab, int ist, int jst) {
  const Basis& ss = c.m.site;
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (twoch_spsm(ti, tj) == 0.0) return 0.0;
  double Si = qn_from_st(ab, ist, 1), Sj = qn_from_st(ab, jst, 1);
  int pos;
  int bi = ss.block_of(ti, pos), bj = ss.block_of(tj, pos);
  double Qt = ss.q(bi, 0), St = ss.q(bi, 1);
  double Scfi = Si - ss.q(bi, 2), Scfj = Sj - ss.q(bj, 2);
  int nsite = (int)std::lround(Qt) + 2;
  double FermiSign = (nsite % 2 == 1) ? -1.0 : 1.0;
  double sigma = Sj - Si;
  double a3 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
  if (dEq(a3, 0.0)) {
    sigma = Si - Sj;
    a3 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (dEq(a3, 0.0)) return 0.0;
  }
  double f = 0.0;
  for (double Szcfj = -Scfj; Szcfj <= Scfj; Szcfj += 1.0) {
    double Szcfi = Szcfj - sigma;
    double Sztj = Sj - Szcfj, Szti = Si - Szcfi;
    if (!dEq(Szti, Sztj) || std::fabs(Sztj) > St) continue;  // the same member, and it exists
    double a0 = c.cg(Scfi, Szcfi, St, Szti, Si, Si);
    double a1 = c.cg(Scfj, Szcfj, St, Sztj, Sj, Sj);
    double a2 = c.cg(Scfi, Szcfi, 0.5, sigma, Scfj, Szcfj);
    f += a0 * a1 * a2 * FermiSign;
  }
  return f / a3;
}

// OneChS_fN_MatEl (OpMatRules.cpp:1555-1654): a spin-1/2 site state is
// looked up as (its (S,Sz) site block) + 1, a missing one giving 0.
double op_f_S(Ctx& c, const Basis& ab, int ist, int jst) {
  const Basis& ss = c.m.site;
  double Si = qn_from_st(ab, ist, 0), Sj = qn_from_st(ab, jst, 0);
  int ti = ab.itype[ist], tj = ab.itype[jst];
  if (ab.stcf[ist] != ab.stcf[jst]) return 0.0;
  double Sti = qn_from_st(ss, ti, 0), Szti = qn_from_st(ss, ti, 1);
  double Stj = qn_from_st(ss, tj, 0), Sztj = qn_from_st(ss, tj, 1);
  double qi[2] = {Sti, Szti}, qj[2] = {Stj, Sztj};
  double Scfi = Si - Szti, Scfj = Sj - Sztj;
  double aux = 0.0, cg1 = 0.0;
  double sigma = Sj - Si;
  for (double Szt = -Stj; Szt <= Stj; Szt += 1.0) {
    qj[1] = Szt;
    int ssj = tj;
    if (tj == 2 || tj == 3) ssj = ss.block_of_qn(qj) + 1;
    qi[1] = Szt - sigma;
    int ssi = ti;
    if (ti == 2 || ti == 3) ssi = ss.block_of_qn(qi) + 1;
    double cg0 = c.cg(Scfi, Si - Szt + sigma, Sti, Szt - sigma, Si, Si);
    cg1 = c.cg(Scfj, Sj - Szt, Stj, Szt, Sj, Sj);
    aux += onechS_fd((int)(sigma / 0.5), ssj, ssi) * cg0 * cg1;
  }
  double n0 = c.cg(Si, Si, 0.5, sigma, Sj, Sj);
  if (!dEq(n0, 0.0)) return aux / n0;
  if (!dEq(cg1, 0.0)) return 0.0 / cg1;
  return 0.0;
}

double op_rule(Ctx& c, int rule, const Basis& ab, int ist, int jst) {
  switch (rule) {
    case R_F_QS: return op_f_QS(c, ab, ist, jst);
    case R_FUP_QSZ: return op_f_QSz(ab, ist, jst, 1);
    case R_FDN_QSZ: return op_f_QSz(ab, ist, jst, -1);
    case R_F1_2CH: return op_f_2ch(c, ab, ist, jst, 1);
    case R_F2_2CH: return op_f_2ch(c, ab, ist, jst, 2);
    case R_IMPONLY: return ab.itype[ist] == ab.itype[jst] ? 1.0 : 0.0;  // ImpOnly_MatEl OpMatRules.cpp:265
    case R_CD_QS: return op_cd_QS(c, ab, ist, jst);
    case R_CD_2CH: return op_cd_2ch(c, ab, ist, jst);
    case R_F_S: return op_f_S(c, ab, ist, jst);
    // OneChSz_fN_MatEl (OpMatRules.cpp:1986-2014)
    case R_FUP_SZ: return ab.stcf[ist] == ab.stcf[jst] ? onechS_fd(1, ab.itype[jst], ab.itype[ist]) : 0.0;
    case R_FDN_SZ: return ab.stcf[ist] == ab.stcf[jst] ? onechS_fd(-1, ab.itype[jst], ab.itype[ist]) : 0.0;
  }
  return 0.0;
}

// ---------------------------------------------------------------- BuildBasis
// BuildBasis (BuildBasis.cpp:8-432) for the Q,S / Q,Sz cases (no parity,
// no symmetry reduction).  befcut: StCameFrom numbers the states before the
// cut (BuildBasis.cpp:386-391), as NRG_main asks when UpdateBefCut = 1.
void build_basis(const Model& m, const Basis& cut, Basis& ab, bool befcut = false) {
  const Basis& ss = m.site;
  int NC = m.common[0];
  std::vector<int> posold(NC), possite(NC), totS(NC, 0), match(NC);
  int its = 0;
  for (int i = 0; i < NC; ++i) {
    posold[i] = m.common[i + 1];
    possite[i] = m.common[i + 1 + NC];
    if (its < (int)m.totS.size() && posold[i] == m.totS[its]) { totS[i] = 1; its++; }
    match[i] = (possite[i] >= 0 && possite[i] < ss.nqn) ? 1 : 0;
  }
  ab = Basis();
  ab.nshell = cut.nshell + 1;
  ab.nqn = NC;
  ab.totalS = !m.totS.empty();
  ab.sqn = m.totS;
  std::vector<double> qo(NC), qs(NC), qnew(NC);
  std::vector<double> cand;
  for (int b = 0; b < cut.nblocks(); ++b) {
    for (int i = 0; i < NC; ++i) qo[i] = cut.q(b, posold[i]);
    for (int s = 0; s < ss.nblocks(); ++s) {
      for (int i = 0; i < NC; ++i) {
        qs[i] = match[i] ? ss.q(s, possite[i]) : 0.0;
        qnew[i] = qs[i] + qo[i];
        cand.push_back(qnew[i]);
      }
      if (!m.totS.empty()) {
        for (int i = 0; i < NC; ++i) {
          if (totS[i] == 1) {
            double Snew = qo[i] + qs[i] - 1.0;
            while (Snew >= std::fabs(qo[i] - qs[i])) {
              qnew[i] = Snew;
              for (int k = 0; k < NC; ++k) cand.push_back(qnew[k]);
              Snew -= 1.0;
            }
          }
        }
      }
    }
  }
  // FilterQNumbers (NRGarrayClass.cpp:271-309): stable removal of exact duplicates.
  std::vector<double>& Q = ab.qn;
  for (size_t k = 0; k < cand.size(); k += NC) {
    bool dup = false;
    for (size_t j = 0; j < Q.size() && !dup; j += NC) {
      bool eq = true;
      for (int i = 0; i < NC && eq; ++i) eq = (Q[j + i] == cand[k + i]);
      dup = eq;
    }
    if (!dup) Q.insert(Q.end(), cand.begin() + k, cand.begin() + k + NC);
  }
  int ist = 0;
  for (int b = 0; b < ab.nblocks(); ++b) {
    for (int i = 0; i < NC; ++i) qnew[i] = ab.q(b, i);
    ab.bbe.push_back(ist);
    for (int bo = 0; bo < cut.nblocks(); ++bo) {
      for (int i = 0; i < NC; ++i) qo[i] = cut.q(bo, posold[i]);
      for (int s = 0; s < ss.nblocks(); ++s) {
        bool ok = true;
        for (int i = 0; i < NC; ++i) {
          qs[i] = match[i] ? ss.q(s, possite[i]) : 0.0;
          if (totS[i] == 0) {
            if (!dEq(qnew[i], qs[i] + qo[i])) ok = false;
          } else {
            double Sold = qo[i], Ssite = ss.q(s, possite[i]), Szsite = ss.q(s, possite[i] + 1);
            if (!dEq(qnew[i], Szsite + Sold) || !triang(Sold, Ssite, qnew[i])) ok = false;
          }
        }
        if (!ok) continue;
        for (int so = cut.bbe[2 * bo]; so <= cut.bbe[2 * bo + 1]; so++)
          for (int st = ss.beg(s); st <= ss.end(s); st++) {
            ab.itype.push_back(ss.itype[st]);
            ab.en.push_back(cut.en[so]);
            ab.stcf.push_back(befcut ? cut.stcf[so] : so);
            ist++;
          }
      }
    }
    ab.bbe.push_back(ist - 1);
  }
}

// ---------------------------------------------------------------- DiagHN
struct Sweep;
double hn_el(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
             int i, int j) {
  switch (c.m.kind) {
    case ORACLE_MODEL_1CHQS: return hn_1chQS(c, P, ab, M, i, j);
    case ORACLE_MODEL_1CHQSZ: return hn_1chQSz(c, P, ab, M, i, j);
    case ORACLE_MODEL_2CHQS: return hn_2chQS(c, P, ab, M, i, j);
    case ORACLE_MODEL_1CHQ: return hn_1chQ(c, P, ab, M, i, j);
    case ORACLE_MODEL_1CHS: return hn_1chS(c, P, ab, M, i, j);
    case ORACLE_MODEL_1CHSZ: return hn_1chSz(c, P, ab, M, i, j);
  }
  return 0.0;
}

template <class F>
void parallel_for(int n, int nthreads, F f) {
  if (nthreads <= 1 || n <= 1) { for (int i = 0; i < n; ++i) f(i); return; }
  std::atomic<int> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < std::min(n, nthreads); ++t)
    th.emplace_back([&]() { for (int i; (i = next.fetch_add(1)) < n;) f(i); });
  for (auto& t : th) t.join();
}

// CNRGmatrix::DiagHN (DiagHN.cpp:6-119) with DiagBlock (NRGmatrixClass.cpp:566-696):
// packed upper triangle, row-major (j >= i), handed to dspev('V','L'); row k
// of the returned Z is eigenvector k.  Optionally keeps the packed blocks.
void diag_hn(Ctx& c, const std::vector<double>& P, const Basis& ab, const std::vector<Mat>& M,
             Arr& eig, int nthreads, std::vector<std::vector<double>>* keepH, double* emin_out) {
  int nb = ab.nblocks();
  std::vector<std::vector<double>> ev(nb), vec(nb), packed(nb);
  // The CG cache is not thread safe: warm it serially on the first row of
  // every block pair type by evaluating the blocks' first element rows.
  auto work = [&](int b, Ctx& cc) {
    int n = ab.bsize(b), b0 = ab.beg(b);
    std::vector<double> A;
    A.reserve((size_t)n * (n + 1) / 2);
    for (int i = 0; i < n; ++i)
      for (int j = i; j < n; ++j) A.push_back(hn_el(cc, P, ab, M, b0 + i, b0 + j));
    if (keepH) packed[b] = A;
    std::vector<double> w(n), Z((size_t)n * n), work3(3 * (size_t)n);
    int info = 0, ldz = n;
    const char jobz = 'V', uplo = 'L';
    g_dspev(&jobz, &uplo, &n, A.data(), w.data(), Z.data(), &ldz, work3.data(), &info, 1, 1);
    ev[b] = w;
    vec[b] = Z;
  };
  if (nthreads <= 1) {
    for (int b = 0; b < nb; ++b) work(b, c);
  } else {
    std::vector<Ctx> ctxs(nthreads, c);
    std::atomic<int> next(0);
    std::vector<std::thread> th;
    for (int t = 0; t < nthreads; ++t)
      th.emplace_back([&, t]() { for (int b; (b = next.fetch_add(1)) < nb;) work(b, ctxs[t]); });
    for (auto& t : th) t.join();
  }
  eig = Arr();
  eig.nshell = ab.nshell; eig.nqn = ab.nqn; eig.qn = ab.qn; eig.bbe = ab.bbe;
  eig.totalS = ab.totalS; eig.sqn = ab.sqn;
  for (int b = 0; b < nb; ++b) {
    eig.en.insert(eig.en.end(), ev[b].begin(), ev[b].end());
    eig.evec.insert(eig.evec.end(), vec[b].begin(), vec[b].end());
  }
  if (keepH) *keepH = packed;
  // SetE0zero (NRGarrayClass.cpp:234-241).
  double emin = *std::min_element(eig.en.begin(), eig.en.end());
  for (double& e : eig.en) e -= emin;
  if (emin_out) *emin_out = emin;
}

// SetDegen (NRGarrayClass.cpp:244-268): pairwise merge of levels closer than
// MyEPS (1e-18), in the reference's order.  Only values with a neighbour
// within MyEPS can change, so the O(n^2) loop runs on those alone.
void set_degen(std::vector<double>& en, double eps) {
  int n = (int)en.size();
  std::vector<int> idx(n);
  for (int i = 0; i < n; ++i) idx[i] = i;
  std::sort(idx.begin(), idx.end(), [&](int a, int b) { return en[a] < en[b]; });
  std::vector<char> cand(n, 0);
  for (int k = 0; k + 1 < n; ++k)
    if (std::fabs(en[idx[k + 1]] - en[idx[k]]) < eps) { cand[idx[k]] = 1; cand[idx[k + 1]] = 1; }
  std::vector<int> list;
  for (int i = 0; i < n; ++i) if (cand[i]) list.push_back(i);
  for (size_t a = 0; a < list.size(); ++a)
    for (size_t b = a + 1; b < list.size(); ++b) {
      int ii = list[a], jj = list[b];
      if (std::fabs(en[jj] - en[ii]) < eps) {
        if (en[jj] > en[ii]) en[jj] = en[ii]; else en[ii] = en[jj];
      }
    }
}

// CNRGarray::Ecut (NRGarrayClass.cpp:661-691).  The window walk stops at the
// end of the spectrum (the reference would read past it).
double ecut(const std::vector<double>& en, int Ncut) {
  std::vector<double> E = en;
  std::sort(E.begin(), E.end());
  size_t sz = E.size();
  if ((size_t)Ncut >= sz - 1) return E.back();
  double aux = E[Ncut - 1], aux2 = E[Ncut];
  size_t ii = 1;
  while ((aux2 > 0.0) && (std::fabs((aux2 - aux) / aux) < 0.01) && (ii < sz) && (Ncut + ii < sz)) {
    aux2 = E[Ncut + ii];
    ii++;
  }
  if (ii > 1) aux = E[Ncut + ii - 2];
  return aux;
}

// SetKept (NRGarrayClass.cpp:461-491).
double set_kept(Arr& a, int Ncut, double eps, int* nkept) {
  set_degen(a.en, eps);
  double ec = ecut(a.en, Ncut);
  a.kept.assign(a.en.size(), 0);
  int nk = 0;
  for (size_t i = 0; i < a.en.size(); ++i) if (a.en[i] <= ec) { a.kept[i] = 1; nk++; }
  if (nkept) *nkept = nk;
  return ec;
}

// CutStates (CutStates.cpp:10-95) with RemoveBlock (NRGarrayClass.cpp:1307)
// and RemoveStatesFromBlock (:1467): whole blocks with E_min > E_cut go, then
// each block loses everything from its first level above E_cut.
void cut_states(const Arr& ain, Basis& acut, int Ncut, double eps) {
  Basis out;
  out.nshell = ain.nshell; out.nqn = ain.nqn; out.totalS = ain.totalS; out.sqn = ain.sqn;
  std::vector<int> eoff(ain.nblocks() + 1, 0);
  for (int b = 0; b < ain.nblocks(); ++b) eoff[b + 1] = eoff[b] + ain.bsize(b) * ain.bsize(b);
  if (Ncut >= ain.nstates()) {
    out.qn = ain.qn; out.bbe = ain.bbe; out.en = ain.en; out.evec = ain.evec; out.kept = ain.kept;
    for (int i = 0; i < ain.nstates(); ++i) out.stcf.push_back(i);
    out.bbe_bc = ain.bbe;
    for (int b = 0; b < ain.nblocks(); ++b) { out.bbe_eig.push_back(eoff[b]); out.bbe_eig.push_back(eoff[b + 1] - 1); }
    acut = out;
    return;
  }
  double ec = ecut(ain.en, Ncut);
  std::vector<double> en = ain.en;  // Acut.SetKept on its own copy
  set_degen(en, eps);
  double ec2 = ecut(en, Ncut);
  std::vector<char> kept(en.size());
  for (size_t i = 0; i < en.size(); ++i) kept[i] = en[i] <= ec2;
  int ist = 0, eig = 0;
  for (int b = 0; b < ain.nblocks(); ++b) {
    int b0 = ain.beg(b), b1 = ain.end(b), n = ain.bsize(b);
    double emin = *std::min_element(en.begin() + b0, en.begin() + b1 + 1);
    if (emin > ec) continue;
    int p = b0;
    while (p <= b1 && en[p] <= ec) p++;   // GetBlockEcutPos (NRGarrayClass.cpp:439-457)
    int k = p - b0;
    for (int q = 0; q < ain.nqn; ++q) out.qn.push_back(ain.q(b, q));
    out.bbe.push_back(ist); out.bbe.push_back(ist + k - 1);
    out.bbe_bc.push_back(b0); out.bbe_bc.push_back(b1);
    for (int i = 0; i < k; ++i) {
      out.en.push_back(en[b0 + i]);
      out.kept.push_back(kept[b0 + i]);
      out.stcf.push_back(b0 + i);
    }
    out.evec.insert(out.evec.end(), ain.evec.begin() + eoff[b], ain.evec.begin() + eoff[b] + (size_t)k * n);
    out.bbe_eig.push_back(eig); out.bbe_eig.push_back(eig + k * n - 1);
    eig += k * n;
    ist += k;
  }
  acut = out;
}

// ---------------------------------------------------------------- UpdateMatrices
// UpdateMatrices (UpdateMatrices.cpp:272-568): for every kept block pair
// allowed by CheckForMatEl and every operator, build fnbasis element by
// element (times the old operator through StCameFrom when NeedOld) and form
// Z_i . fnbasis . Z_j^T with two dgemm calls.
void update_matrices(Ctx& c, const Basis& acut, const Basis& ab, std::vector<Mat>& mats, int nthreads) {
  std::vector<Mat> old = mats;
  // FindMatchBlock (FindMatchBlock.cpp:5-24).
  std::vector<int> bc(acut.nblocks());
  for (int b = 0; b < acut.nblocks(); ++b) bc[b] = ab.block_of_qn(&acut.qn[(size_t)b * acut.nqn]);
  for (size_t im = 0; im < mats.size(); ++im) {
    Mat& M = mats[im];
    M.clear_data();
    M.blk = acut;
    M.blk.evec.clear();
    struct Job { int i, j; };
    std::vector<Job> jobs;
    for (int i = 0; i < acut.nblocks(); ++i)
      for (int j = 0; j < acut.nblocks(); ++j)
        if (check(c.m.op_check[im], acut, i, j)) jobs.push_back({i, j});
    std::vector<std::vector<double>> res(jobs.size());
    auto work = [&](int k, Ctx& cc) {
      int i = jobs[k].i, j = jobs[k].j;
      int ni = acut.bsize(i), nj = acut.bsize(j);
      int ib = bc[i], jb = bc[j];
      int niBC = ab.bsize(ib), njBC = ab.bsize(jb);
      std::vector<double> F((size_t)niBC * njBC);
      size_t r = 0;
      for (int ist = ab.beg(ib); ist <= ab.end(ib); ist++)
        for (int jst = ab.beg(jb); jst <= ab.end(jb); jst++) {
          double v = op_rule(cc, c.m.op_rule[im], ab, ist, jst);
          if (M.need_old) v = v * old[im].get(ab.stcf[ist], ab.stcf[jst]);
          F[r++] = v;
        }
      const double* Zi = &acut.evec[acut.bbe_eig[2 * i]];
      const double* Zj = &acut.evec[acut.bbe_eig[2 * j]];
      std::vector<double> T((size_t)niBC * nj), O((size_t)ni * nj);
      g_dgemm(kRowMajor, kNoTrans, kTrans, niBC, nj, njBC, 1.0, F.data(), njBC, Zj, njBC, 0.0, T.data(), nj);
      g_dgemm(kRowMajor, kNoTrans, kNoTrans, ni, nj, niBC, 1.0, Zi, niBC, T.data(), nj, 0.0, O.data(), nj);
      res[k] = O;
    };
    if (nthreads <= 1) {
      for (size_t k = 0; k < jobs.size(); ++k) work((int)k, c);
    } else {
      std::vector<Ctx> ctxs(nthreads, c);
      std::atomic<int> next(0);
      std::vector<std::thread> th;
      for (int t = 0; t < nthreads; ++t)
        th.emplace_back([&, t]() { for (int k; (k = next.fetch_add(1)) < (int)jobs.size();) work(k, ctxs[t]); });
      for (auto& t : th) t.join();
    }
    for (size_t k = 0; k < jobs.size(); ++k)
      M.push_block(jobs[k].i, jobs[k].j, res[k].data(), (int)res[k].size());
  }
}

// ---------------------------------------------------------------- observables
// CalcSuscep (CalcThermo.cpp:16-74): returns <Sz^2>/Z (the <Sz>^2 term is
// multiplied by 0 in the reference).
double calc_suscep(const Arr& a, double beta, int sq, bool totalS) {
  if (sq < 0) return 0.0;  // Sqnumber -1 ("no spin whatsoever"): not taken by the reference
  double s0 = 0, s1 = 0, s2 = 0;
  for (int b = 0; b < a.nblocks(); ++b) {
    double Si = a.q(b, sq);
    for (int i = a.beg(b); i <= a.end(b); i++) {
      double auxS, SzSq, Sz;
      if (totalS) { auxS = 2.0 * Si + 1.0; SzSq = (1.0 / 12.0) * auxS * (auxS * auxS - 1.0); Sz = 0.0; }
      else { auxS = 1.0; SzSq = Si * Si; Sz = Si; }
      double e = std::exp(-beta * a.en[i]);
      s0 += auxS * e; s1 += SzSq * e; s2 += Sz * e;
    }
  }
  return (s1 - 0.0 * s1 * s2) / s0;
}
// CalcEntropy (CalcThermo.cpp:80-121).
double calc_entropy(const Arr& a, double beta, int sq, bool totalS) {
  double Z = 0, s = 0;
  for (int b = 0; b < a.nblocks(); ++b) {
    double deg = totalS ? 2.0 * a.q(b, sq) + 1.0 : 1.0;
    for (int i = a.beg(b); i <= a.end(b); i++) {
      double E = a.en[i], e = std::exp(-beta * E);
      s += deg * E * e; Z += deg * e;
    }
  }
  return beta * (s / Z) + std::log(Z);
}
// CalcOpAvg (CalcOpAvg.cpp:13-84): Boltzmann average of a diagonal operator
// over the kept states.
double calc_opavg(const Arr& a, const Mat& M, double beta, bool totalS, int sq) {
  double s = 0, Z = 0;
  for (int b = 0; b < a.nblocks(); ++b) {
    double deg = totalS ? 2.0 * a.q(b, sq) + 1.0 : 1.0;
    for (int i = a.beg(b); i <= a.end(b); i++) {
      double e = std::exp(-beta * a.en[i]);
      s += deg * M.get(i, i) * e; Z += deg * e;
    }
  }
  if (!(std::fabs(Z - 0.0) < 1.e-20)) s = s / Z;
  return s;
}

// ---------------------------------------------------------------- model set-up
// Operator matrix on one-state-per-block arrays.
Mat diag_op(const Arr& a, const std::vector<double>& vals, const char* name) {
  Mat M; M.blk = a; M.blk.evec.clear(); M.need_old = true; M.calc_avg = true; M.name = name;
  M.rule = R_IMPONLY;
  for (int b = 0; b < a.nblocks(); ++b) { double v = vals[b]; M.push_block(b, b, &v, 1); }
  return M;
}

// OneChQS_SetAnderson_Hm1 (Main/Main_SetH0.cpp:1794-1969): three impurity
// multiplets, reduced <||d||> = (1, -sqrt 2), n_d, n_d^2 and S^2.
void hm1_QS(double Lambda, double HLF, double U, double ed, Arr& a, Mat& f, std::vector<Mat>& avg) {
  a = Arr(); a.nqn = 2; a.nshell = -1; a.totalS = true; a.sqn = {1};
  a.qn = {-1, 0, 0, 0.5, 1, 0};
  a.bbe = {0, 0, 1, 1, 2, 2};
  a.en = {0.5 * U / (Lambda * HLF), (ed + 0.5 * U) / (Lambda * HLF), (2.0 * ed + 1.5 * U) / (Lambda * HLF)};
  a.evec = {1, 1, 1};
  f = Mat(); f.blk = a; f.blk.evec.clear();
  double one = 1.0, m2 = -std::sqrt(2.0);
  f.push_block(0, 1, &one, 1); f.push_block(1, 2, &m2, 1);
  std::vector<double> nd, nd2, s2;
  for (int b = 0; b < 3; ++b) {
    double n = a.q(b, 0) + 1.0, S = a.q(b, 1);
    nd.push_back(n); nd2.push_back(n * n); s2.push_back(S * (S + 1.0));
  }
  avg = {diag_op(a, nd, "Ndot"), diag_op(a, nd2, "NdSq"), diag_op(a, s2, "SdSq")};
}

// OneChQSz_SetAnderson_Hm1 (Main/Main_SetH0.cpp:421-660): four impurity
// states, f_up, f_dn, n_d and S_z.
void hm1_QSz(double Lambda, double HLF, double U, double ed, double B, Arr& a, Mat& fu, Mat& fd,
             std::vector<Mat>& avg) {
  double hz = 0.5 * B;
  a = Arr(); a.nqn = 2; a.nshell = -1; a.totalS = false;
  a.qn = {-1, 0, 0, 0.5, 0, -0.5, 1, 0};
  a.bbe = {0, 0, 1, 1, 2, 2, 3, 3};
  a.en = {0.5 * U / (Lambda * HLF), (ed + 0.5 * U - hz) / (Lambda * HLF), (ed + 0.5 * U + hz) / (Lambda * HLF),
          (2.0 * ed + 1.5 * U) / (Lambda * HLF)};
  a.evec = {1, 1, 1, 1};
  double one = 1.0, mone = -1.0;
  fu = Mat(); fu.blk = a; fu.blk.evec.clear();
  fu.push_block(0, 1, &one, 1); fu.push_block(2, 3, &one, 1);
  fd = Mat(); fd.blk = a; fd.blk.evec.clear();
  fd.push_block(0, 2, &one, 1); fd.push_block(1, 3, &mone, 1);
  std::vector<double> nd, sz;
  for (int b = 0; b < 4; ++b) { nd.push_back(a.q(b, 0) + 1.0); sz.push_back(a.q(b, 1)); }
  avg = {diag_op(a, nd, "Ndot"), diag_op(a, sz, "Szdot")};
}

// TwoChQS_SetH0Chain (Main/Main_SetH0.cpp:3472-3560): the two-channel first
// site in its multiplet basis (QNumbers, BlockBegEnd and iType as listed
// there, StCameFrom 0, all energies 0, identity eigenvectors), and f_ch1,
// f_ch2 by CNRGmatrix::SetMatrix (NRGmatrixClass.cpp:1836-1877): every block
// pair passing CheckForMatEl, every state pair through CalcMatEl.
void h0_chain_2chQS(Ctx& c, Arr& a, Mat& f1, Mat& f2) {
  Basis b; b.nqn = 2; b.nshell = 0;
  b.qn = {-2, 0, -1, 0.5, 0, 0, 0, 1, 1, 0.5, 2, 0};
  b.bbe = {0, 0, 1, 2, 3, 5, 6, 6, 7, 8, 9, 9};
  b.itype = {0, 1, 2, 5, 6, 7, 10, 11, 12, 15};
  b.stcf.assign(10, 0);
  a = Arr(); a.nqn = 2; a.nshell = 0; a.totalS = true; a.sqn = {1};
  a.qn = b.qn; a.bbe = b.bbe;
  a.en.assign(10, 0.0);
  for (int k = 0; k < a.nblocks(); ++k)
    for (int i = 0; i < a.bsize(k); ++i)
      for (int j = 0; j < a.bsize(k); ++j) a.evec.push_back(i == j ? 1.0 : 0.0);
  Mat* out[2] = {&f1, &f2};
  const int rules[2] = {R_F1_2CH, R_F2_2CH};
  for (int o = 0; o < 2; ++o) {
    Mat& M = *out[o];
    M = Mat(); M.blk = a; M.blk.evec.clear();
    for (int i = 0; i < b.nblocks(); ++i)
      for (int j = 0; j < b.nblocks(); ++j) {
        if (!check(C_2CH_CD, b, i, j)) continue;
        std::vector<double> v;
        for (int ist = b.beg(i); ist <= b.end(i); ++ist)
          for (int jst = b.beg(j); jst <= b.end(j); ++jst) v.push_back(op_rule(c, rules[o], b, ist, jst));
        M.push_block(i, j, v.data(), (int)v.size());
      }
  }
}

// OneChS_SetAnderson_Hm1 (Main/Main_SetH0.cpp:2618-2738): S blocks 0
// (|0>, |up dn>) and 1/2; reduced f; n_d, n_d^2, S^2 on the diagonal.
void hm1_S(double Lambda, double HLF, double U, double ed, Arr& a, Mat& f, std::vector<Mat>& avg) {
  a = Arr(); a.nqn = 1; a.nshell = -1; a.totalS = true; a.sqn = {0};
  a.qn = {0.0, 0.5};
  a.bbe = {0, 1, 2, 2};
  a.en = {0.5 * U / (Lambda * HLF), (2.0 * ed + 1.5 * U) / (Lambda * HLF), (ed + 0.5 * U) / (Lambda * HLF)};
  a.evec = {1, 0, 0, 1, 1};
  f = Mat(); f.blk = a; f.blk.evec.clear();
  const double f01[2] = {1.0, 0.0}, f10[2] = {0.0, -std::sqrt(2.0)};
  f.push_block(0, 1, f01, 2); f.push_block(1, 0, f10, 2);
  Mat nd, nd2, s2;
  for (Mat* m : {&nd, &nd2, &s2}) { m->blk = a; m->blk.evec.clear(); }
  nd.name = "Ndot"; nd2.name = "NdSq"; s2.name = "SdSq";
  const double n0[4] = {0, 0, 0, 2}, n1[1] = {1}, q0[4] = {0, 0, 0, 4}, q1[1] = {1}, s0[4] = {0, 0, 0, 0},
               s1[1] = {0.75};
  nd.push_block(0, 0, n0, 4); nd.push_block(1, 1, n1, 1);
  nd2.push_block(0, 0, q0, 4); nd2.push_block(1, 1, q1, 1);
  s2.push_block(0, 0, s0, 4); s2.push_block(1, 1, s1, 1);
  avg = {nd, nd2, s2};
}

// OneChSz_SetAnderson_Hm1 (Main/Main_SetH0.cpp:2751-2933): Sz blocks 0
// (|0>, |up dn>), +1/2, -1/2, Zeeman -hz S_z with hz = B/2; f_up, f_dn;
// matrices 2..4 named Ndot, NdSq, SdSq hold n_d, S_z, S_z^2.
void hm1_Sz(double Lambda, double HLF, double U, double ed, double B, Arr& a, Mat& fu, Mat& fd,
            std::vector<Mat>& avg) {
  const double hz = 0.5 * B;
  a = Arr(); a.nqn = 1; a.nshell = -1; a.totalS = false;
  a.qn = {0.0, 0.5, -0.5};
  a.bbe = {0, 1, 2, 2, 3, 3};
  a.en = {0.5 * U / (Lambda * HLF), (2.0 * ed + 1.5 * U) / (Lambda * HLF), (ed + 0.5 * U - hz) / (Lambda * HLF),
          (ed + 0.5 * U + hz) / (Lambda * HLF)};
  a.evec = {1, 0, 0, 1, 1, 1};
  fu = Mat(); fu.blk = a; fu.blk.evec.clear();
  fd = Mat(); fd.blk = a; fd.blk.evec.clear();
  const double u01[2] = {1, 0}, u20[2] = {0, 1}, d02[2] = {1, 0}, d10[2] = {0, -1};
  fu.push_block(0, 1, u01, 2); fu.push_block(2, 0, u20, 2);
  fd.push_block(0, 2, d02, 2); fd.push_block(1, 0, d10, 2);
  Mat nd, sz, sz2;
  for (Mat* m : {&nd, &sz, &sz2}) { m->blk = a; m->blk.evec.clear(); }
  nd.name = "Ndot"; sz.name = "NdSq"; sz2.name = "SdSq";
  const double n0[4] = {0, 0, 0, 2}, one[1] = {1}, z0[4] = {0, 0, 0, 0}, zp[1] = {0.5}, zm[1] = {-0.5},
               q[1] = {0.25};
  nd.push_block(0, 0, n0, 4); nd.push_block(1, 1, one, 1); nd.push_block(2, 2, one, 1);
  sz.push_block(0, 0, z0, 4); sz.push_block(1, 1, zp, 1); sz.push_block(2, 2, zm, 1);
  sz2.push_block(0, 0, z0, 4); sz2.push_block(1, 1, q, 1); sz2.push_block(2, 2, q, 1);
  avg = {nd, sz, sz2};
}

// OneChQ_SetAnderson_Hm1 (Main/Main_SetH0.cpp:217-352): one quantum number,
// the Q = 0 block holds |up>, |dn>; f_up, f_dn not reduced; S_z and S_z^2
// from iDegen/10 on the diagonal.
void hm1_Q(double Lambda, double HLF, double U, double ed, Arr& a, Mat& fu, Mat& fd, std::vector<Mat>& avg) {
  a = Arr(); a.nqn = 1; a.nshell = -1; a.totalS = false;
  a.qn = {-1, 0, 1};
  a.bbe = {0, 0, 1, 2, 3, 3};
  a.en = {0.5 * U / (Lambda * HLF), (ed + 0.5 * U) / (Lambda * HLF), (ed + 0.5 * U) / (Lambda * HLF),
          (2.0 * ed + 1.5 * U) / (Lambda * HLF)};
  a.evec = {1, 1, 0, 0, 1, 1};
  fu = Mat(); fu.blk = a; fu.blk.evec.clear();
  fd = Mat(); fd.blk = a; fd.blk.evec.clear();
  const double u01[2] = {1, 0}, u12[2] = {0, 1}, d01[2] = {0, 1}, d12[2] = {-1, 0};
  fu.push_block(0, 1, u01, 2); fu.push_block(1, 2, u12, 2);
  fd.push_block(0, 1, d01, 2); fd.push_block(1, 2, d12, 2);
  Mat sz, sz2;
  sz.blk = a; sz.blk.evec.clear(); sz.name = "Sz";
  sz2.blk = a; sz2.blk.evec.clear(); sz2.name = "Sz2";
  const double z0[1] = {0}, z1[4] = {0.5, 0, 0, -0.5}, q1[4] = {0.25, 0, 0, 0.25};
  sz.push_block(0, 0, z0, 1); sz.push_block(1, 1, z1, 4); sz.push_block(2, 2, z0, 1);
  sz2.push_block(0, 0, z0, 1); sz2.push_block(1, 1, q1, 4); sz2.push_block(2, 2, z0, 1);
  avg = {sz, sz2};
}

// ---------------------------------------------------------------- DM-NRG
// What NRG_main saves per shell when the spectral density is asked for
// (calcdens = 1, UpdateBefCut = 1; CNRGCodeHandler::SaveArrays,
// NRGcodehandlerClass.cpp:887-932): Abasis_N, the uncut eigen-array Acut_N
// (all states, Kept flags, all eigenvectors) and the c_d operator in it.
struct DmShell {
  Basis ab;
  Basis full;
  Mat cd;
};

// CalcDN (CalcDN.cpp) with z = 1.
double calc_dn(double L, int N) {
  double hlf = L > 0.0 ? 0.5 * (1.0 + (1.0 / L)) : 1.0;
  return hlf * std::pow(L, (-(N - 1) / 2.0) - 1.0 + 1.0);
}
// LogGaussDelta (BroadDelta.cpp:116-133) and GaussDelta (BroadDelta.cpp:96-106).
double log_gauss_delta(double omega, double Ep, double b) {
  if (Ep == 0.0) Ep = 1.0E-100;
  if ((omega * Ep) < 0.0) return 0.0;
  double a0 = 1.0 / (b * std::fabs(Ep) * std::sqrt(3.141592653589793238462643383279502884197169));
  double a1 = std::log(std::fabs(omega / Ep)) / b;
  return a0 * std::exp(-(a1 - b / 4.0) * (a1 - b / 4.0));
}
double gauss_delta(double omega, double Ep, double b) {
  double a0 = 1.0 / (b * std::sqrt(3.141592653589793238462643383279502884197169));
  double a1 = (omega - Ep) / b;
  return a0 * std::exp(-a1 * a1);
}
// PartitionFunc / PartitionFuncDisc (NRGarrayClass.cpp:997-1060): (2S+1)
// weighted Boltzmann sums over all / discarded states.
double partition(const Arr& a, double beta, bool disc_only) {
  double sum = 0.0;
  for (int b = 0; b < a.nblocks(); ++b) {
    double Si = a.totalS ? a.q(b, a.sqn[0]) : 0.0;
    for (int i = a.beg(b); i <= a.end(b); ++i)
      if (!disc_only || !a.kept[i]) sum += (2.0 * Si + 1.0) * std::exp(-beta * a.en[i]);
  }
  return sum;
}

struct DmParams {
  double lambda, temp, betabar, bbroad, twindow, broadtemp, site_dim;
  double tempbar0;  // TempBar handed to DM_NRG_SetRhoNmax
};

// DM_NRG's temperature (DM_NRG.cpp:100-121): Mtemp < Nsitesmax-1 puts T at
// D_Mtemp/betabar, otherwise at D_{Nsitesmax+199}/betabar; a positive
// `temp` given by the caller replaces the latter.  SetRhoNmax receives
// T/D_Mtemp or T/D_{Nsitesmax-1} respectively.
void dm_temperature(DmParams& p, int nsites, int mtemp, double temp) {
  const double L = p.lambda;
  if (mtemp >= 0 && mtemp < nsites - 1) {
    double DM = calc_dn(L, mtemp);
    p.temp = DM / p.betabar;
    p.tempbar0 = p.temp / DM;
  } else {
    p.temp = temp > 0.0 ? temp : calc_dn(L, nsites + 199) / p.betabar;
    p.tempbar0 = p.temp / calc_dn(L, nsites - 1);
  }
}

// Dense symmetric density-matrix blocks, one per block of the uncut array.
typedef std::vector<std::vector<double>> RhoBlocks;

// DM_NRG main (DM_NRG/DM_NRG.cpp:128-383) for the default temperature branch
// (Mtemp >= Nsitesmax-1) with FDM: partition sums, DM_NRG_SetRhoNmax
// (DM_NRG_SetRhoNmax.cpp:9-126) and, shell by shell, RotateMatrix
// (RotateMatrix.cpp:17-99) + DM_NRG_CalcRhoN_withSU2 (DM_NRG_CalcRhoN.cpp:252-449).
// site_dim is the 4.0 of DM_NRG.cpp:292 (d of one Wilson site).
void dm_backward(Ctx& c, const std::vector<DmShell>& sh, const DmParams& p, std::vector<RhoBlocks>& rho) {
  const int nsites = (int)sh.size();
  const int Nmax = nsites - 1;
  const double L = p.lambda, Temp = p.temp;
  const double TempBar0 = p.tempbar0;
  double DM = calc_dn(L, Nmax - 1);
  double TempBar = Temp / DM;
  double ZTot = partition(sh[Nmax].full, 1.0 / TempBar, false);
  for (int N = Nmax - 1; N >= 0; --N) {
    DM = calc_dn(L, N - 1);
    TempBar = Temp / DM;
    double ZNdisc = partition(sh[N].full, 1.0 / TempBar, true);
    ZTot += ZNdisc * std::pow(p.site_dim, Nmax - N);
  }
  rho.assign(nsites, RhoBlocks());
  {  // SetRhoNmax
    const Arr& a = sh[Nmax].full;
    double beta = dEq(TempBar0, 0.0) ? 1.0e10 : 1.0 / TempBar0;
    rho[Nmax].resize(a.nblocks());
    for (int b = 0; b < a.nblocks(); ++b) {
      int n = a.bsize(b);
      std::vector<double>& R = rho[Nmax][b];
      R.assign((size_t)n * n, 0.0);
      for (int i = 0; i < n; ++i) R[(size_t)i * n + i] = std::exp(-beta * a.en[a.beg(b) + i]) / ZTot;
    }
  }
  for (int N = Nmax - 1; N >= 0; --N) {
    const Arr& aN = sh[N].full;
    const Basis& fNp1 = sh[N + 1].full;
    const Basis& abNp1 = sh[N + 1].ab;
    DM = calc_dn(L, N - 1);
    TempBar = Temp / DM;
    const double ZNdisc = ZTot / std::pow(p.site_dim, Nmax - N);
    const double beta = 1 / TempBar;
    // RotateMatrix: rho~ = Z^T rho Z per block, in the before-cut basis.
    RhoBlocks rot(fNp1.nblocks());
    for (int b = 0; b < fNp1.nblocks(); ++b) {
      int n = fNp1.bsize(b), nb = fNp1.bsize_bc(b);
      const double* Z = &fNp1.evec[fNp1.bbe_eig[2 * b]];
      const std::vector<double>& R = rho[N + 1][b];
      std::vector<double> T((size_t)n * nb, 0.0);
      for (int i = 0; i < n; ++i)
        for (int j = 0; j < nb; ++j) {
          double s = 0.0;
          for (int k = 0; k < n; ++k) s += R[(size_t)i * n + k] * Z[(size_t)k * nb + j];
          T[(size_t)i * nb + j] = s;
        }
      std::vector<double>& O = rot[b];
      O.assign((size_t)nb * nb, 0.0);
      for (int i = 0; i < nb; ++i)
        for (int j = 0; j < nb; ++j) {
          double s = 0.0;
          for (int k = 0; k < n; ++k) s += Z[(size_t)k * nb + i] * T[(size_t)k * nb + j];
          O[(size_t)i * nb + j] = s;
        }
    }
    // DM_NRG_SetChildSt (DM_NRG_SetChildSt.cpp:11-40).
    std::vector<std::vector<int>> child(aN.nstates());
    for (size_t k = 0; k < abNp1.stcf.size(); ++k) child[abNp1.stcf[k]].push_back((int)k);
    rho[N].resize(aN.nblocks());
    for (int b = 0; b < aN.nblocks(); ++b) {
      int n = aN.bsize(b), b0 = aN.beg(b);
      double Sold = aN.totalS ? aN.q(b, aN.sqn[0]) : 0.0;
      std::vector<double>& R = rho[N][b];
      R.assign((size_t)n * n, 0.0);
      for (int i = 0; i < n; ++i)
        for (int j = i; j < n; ++j) {
          int ist = b0 + i, jst = b0 + j;
          double v = 0.0;
          // DM_NRG_SetChildSameType (DM_NRG_SetChildSt.cpp:45-113).
          for (int ci : child[ist]) {
            int pos;
            int ib = abNp1.block_of(ci, pos);
            int ti = abNp1.itype[ci];
            for (int cj : child[jst]) {
              int jb = abNp1.block_of(cj, pos);
              if (ti != abNp1.itype[cj] || ib != jb) continue;
              double Si = abNp1.totalS ? abNp1.q(ib, abNp1.sqn[0]) : 0.0;
              const int tb = c.m.site.block_of(ti, pos);
              double St = c.m.site.totalS ? c.m.site.q(tb, c.m.site.sqn[0]) : 0.0;
              double cgf = 0.0;
              for (double Sz = -Si; Sz <= Si; Sz += 1.0) {
                double x = c.cg(Sold, Sold, St, Sz - Sold, Si, Sz);
                cgf += x * x;
              }
              int nb = fNp1.bsize_bc(ib);
              int pi = ci - fNp1.bbe_bc[2 * ib], pj = cj - fNp1.bbe_bc[2 * ib];
              v += cgf * rot[ib][(size_t)pi * nb + pj];
            }
          }
          if (i == j && !aN.kept[ist] && !dEq(ZNdisc, 0.0)) v = std::exp(-beta * (aN.en[ist])) / ZNdisc;
          R[(size_t)i * n + j] = v;
          R[(size_t)j * n + i] = v;
        }
    }
  }
}

// CSpecFunction::MijxBDeltaEij (SpecFunc_allSTL.cpp:132-220 and
// SpecFuncClass.cpp:934-990): the broadened delta between two levels, the
// log-Gaussian, or a Gaussian inside the thermal window.
double broad_delta(const DmParams& p, double omega, double dE, double TempDN) {
  double BD = log_gauss_delta(omega, dE, p.bbroad);
  if (std::fabs(dE) < p.twindow * TempDN) BD = gauss_delta(omega, dE, p.broadtemp);
  return BD;
}

// Sum_{Sz} <S1 Sz; 1/2 1/2 | S2 Sz+1/2>^2 of the spectral sums
// (SpecFunc_allSTL.cpp, end of FDM_SpecDens_M_STL; SpecFuncClass.cpp:600-617).
double spec_cg(Ctx& c, const Arr& a, int b1, int b2) {
  if (!a.totalS) return 1.0;
  double S1 = a.q(b1, a.sqn[0]), S2 = a.q(b2, a.sqn[0]), f = 0.0;
  for (double Sz1 = -S1; Sz1 <= S1; Sz1 += 1.0) {
    double x = c.cg(S1, Sz1, 0.5, 0.5, S2, Sz1 + 0.5);
    f += x * x;
  }
  return f;
}

// CSpecFunction::CalcSpecCosti_T_N (SpecFuncClass.cpp:417-650): the last shell.
double spec_costi(Ctx& c, const DmShell& s, int N, const DmParams& p, double omegabar) {
  const Arr& a = s.full;
  const Mat& A = s.cd;
  const double TempDN = p.temp / calc_dn(p.lambda, N);
  double rho = 0.0;
  for (size_t k = 0; k < A.map.size() / 2; ++k) {
    int b1 = A.map[2 * k], b2 = A.map[2 * k + 1];
    int n1 = a.bsize(b1), n2 = a.bsize(b2), o1 = a.beg(b1), o2 = a.beg(b2);
    const double* M = &A.el[A.mbe[2 * k]];
    double tr = 0.0;
    for (int bb = 0; bb < n2; ++bb)
      for (int aa = 0; aa < n1; ++aa) {
        double E1 = a.en[o1 + aa], E2 = a.en[o2 + bb];
        double m = M[(size_t)aa * n2 + bb];
        double sum12 = m * std::exp(-p.betabar * E1) + std::exp(-p.betabar * E2) * m;
        tr += sum12 * (m * broad_delta(p, omegabar, E2 - E1, TempDN));
      }
    rho += spec_cg(c, a, b1, b2) * tr;
  }
  return rho / partition(a, p.betabar, false);
}

// CSpecFunction::FDM_SpecDens_M_STL (SpecFunc_allSTL.cpp:1253-2358), real
// operators, Op2 = Op1.  Each term is the trace of (B^T rho or rho B^T) times
// A o delta over one kept/discarded sub-block pair.
double spec_fdm(Ctx& c, const std::vector<DmShell>& sh, const std::vector<RhoBlocks>& rho, int N,
                const DmParams& p, double omegabar) {
  const int nshell = (int)sh.size();
  if (N > nshell - 1) return 0.0;
  if (N == nshell - 1) {
    // FDM_SpecDens_M_STL sets Betabar = 1e10 when Temp is zero within 1e-20.
    DmParams q = p;
    if (dEq(p.temp, 0.0)) q.betabar = 1.0e10;
    return spec_costi(c, sh[N], N, q, omegabar);
  }
  const Arr& a = sh[N].full;
  const Mat& A = sh[N].cd;
  const double TempDN = p.temp / calc_dn(p.lambda, N);
  double pos_w = 0.0, neg_w = 0.0;
  for (size_t k = 0; k < A.map.size() / 2; ++k) {
    int b1 = A.map[2 * k], b2 = A.map[2 * k + 1];
    int n1 = a.bsize(b1), n2 = a.bsize(b2), o1 = a.beg(b1), o2 = a.beg(b2);
    std::vector<int> K1, D1, K2, D2;
    for (int i = 0; i < n1; ++i) (a.kept[o1 + i] ? K1 : D1).push_back(i);
    for (int i = 0; i < n2; ++i) (a.kept[o2 + i] ? K2 : D2).push_back(i);
    if ((K1.empty() && K2.empty()) || (D1.empty() && D2.empty())) continue;
    const double* M = &A.el[A.mbe[2 * k]];
    const std::vector<double>& R1 = rho[N][b1];
    const std::vector<double>& R2 = rho[N][b2];
    auto el = [&](int i, int j) { return M[(size_t)i * n2 + j]; };
    auto bd = [&](int i, int j) { return broad_delta(p, omegabar, a.en[o2 + j] - a.en[o1 + i], TempDN); };
    // trace over b in S2 of sum_{a in S1} (sum_{a' in S1} A[a',b] rho1[a',a]) A[a,b] d(a,b)
    auto term1 = [&](const std::vector<int>& S1, const std::vector<int>& S2) {
      double t = 0.0;
      for (int bb : S2)
        for (int aa : S1) {
          double pr = 0.0;
          for (int ap : S1) pr += el(ap, bb) * R1[(size_t)ap * n1 + aa];
          t += pr * (el(aa, bb) * bd(aa, bb));
        }
      return t;
    };
    // trace over b in S2 of sum_{a in S1} (sum_{b' in S2} rho2[b,b'] A[a,b']) A[a,b] d(a,b)
    auto term2 = [&](const std::vector<int>& S1, const std::vector<int>& S2) {
      double t = 0.0;
      for (int bb : S2)
        for (int aa : S1) {
          double pr = 0.0;
          for (int bp : S2) pr += R2[(size_t)bb * n2 + bp] * el(aa, bp);
          t += pr * (el(aa, bb) * bd(aa, bb));
        }
      return t;
    };
    double T1KK = 0, T1DDADD = 0, T1DDADK = 0, T2KK = 0, T2DDADD = 0, T2DDAKD = 0;
    if (!K1.empty() && !D2.empty() && omegabar >= 0.0) T1KK = term1(K1, D2);
    if (!D1.empty() && !D2.empty()) {
      T1DDADD = term1(D1, D2);
      if (!K2.empty()) T1DDADK = term1(D1, K2);
    }
    if (!D1.empty() && !K2.empty() && omegabar < 0.0) T2KK = term2(D1, K2);
    if (!D1.empty() && !D2.empty()) {
      T2DDADD = term2(D1, D2);
      if (!K1.empty()) T2DDAKD = term2(K1, D2);
    }
    double cgf = spec_cg(c, a, b1, b2);
    pos_w += cgf * (T1KK + T1DDADD + T2DDADD + T2DDAKD);
    neg_w += cgf * (T2KK + T1DDADD + T1DDADK + T2DDADD);
  }
  return omegabar >= 0.0 ? pos_w : neg_w;
}

// CSpecFunction::CalcNfromOmega (SpecFuncClass.cpp:41-49) and CalcSpecDM_NRG
// (SpecFuncClass.cpp:1827-1883): the shells within a window around omega.
double spec_at(Ctx& c, const std::vector<DmShell>& sh, const std::vector<RhoBlocks>& rho, const DmParams& p,
               double omega) {
  const double L = p.lambda, hlf = 0.5 * (1.0 + (1.0 / L));
  const int nshell = (int)sh.size();
  int iaux = (int)(2.0 * std::log(2.0 * std::fabs(omega) / hlf) / std::log(L));
  iaux = 1 - iaux;
  if (iaux < 0) iaux = 0;
  int N0 = iaux - 8 > 0 ? iaux - 8 : 0;
  int N1 = iaux + 14 < nshell ? iaux + 14 : nshell;
  double s = 0.0;
  for (int N = N0; N < N1; ++N) {
    double DN = calc_dn(L, N);
    s += spec_fdm(c, sh, rho, N, p, omega / DN) / DN;
  }
  return s;
}

// CSpecFunction::CalcSpec_ManyOmegas (SpecFuncClass.cpp:2238-2341), FDM:
// nw frequencies per shell from shell 2 to the last-but-one, negative side
// first.
void spec_grid(double L, int nshell, int nw, std::vector<double>& om) {
  const double hlf = 0.5 * (1.0 + (1.0 / L)), factorWN = std::pow(L, 1.25);
  auto dn = [&](int N) { return hlf * std::pow(L, (-(N - 1) / 2.0) - 1.0 + 1.0); };
  const int Nmax = nshell - 1, N0 = 2;
  om.clear();
  for (int N = N0; N <= Nmax; ++N) {
    double WN = factorWN * dn(N);
    for (int i = 0; i < nw; ++i) om.push_back(-(std::pow(L, -((double)i / (2.0 * nw))) * WN));
  }
  for (int N = Nmax; N >= N0; --N) {
    double WN = factorWN * dn(N);
    for (int i = nw - 1; i >= 0; --i) om.push_back(std::pow(L, -((double)i / (2.0 * nw))) * WN);
  }
}

}  // namespace

// ================================================================ C ABI
struct OracleIter {
  std::vector<double> params;     // ParamsHN used for this iteration
  std::vector<double> qn;         // block QNs
  std::vector<int> bsize;         // block sizes
  std::vector<double> en;         // energies after SetE0zero + SetDegen
  double emin = 0, ecut = 0;
  int nkept = 0;
  std::vector<double> thermo;     // 4 x (beta, T, suscep, entropy)
  std::vector<double> opavg;      // CalcAvg operators over AeigCut
  std::vector<int> kept_bsize;    // AeigCut block sizes
  double seconds = 0;             // wall time of this iteration
  // Optional capture of the DiagHN inputs/outputs for drop-in tests.
  std::vector<double> basis_qn, basis_en;
  std::vector<int> basis_bbe, basis_itype, basis_stcf;
  std::vector<double> H;          // packed upper triangles, block-concatenated
  // Every input and output of the iteration's DiagHN / SetKept / CutStates /
  // UpdateMatrices steps, by name (see oracle_run).
  std::map<std::string, std::vector<double>> capd;
  std::map<std::string, std::vector<int>> capi;
};

struct OracleRun {
  int nqn = 2;
  int model = 0;
  double lambda = 2.5;
  std::vector<DmShell> dm;        // per shell, when cfg->dm is set
  std::vector<double> opavg_m1;
  std::vector<std::string> opnames;
  std::vector<OracleIter> it;
  double seconds = 0;
};

extern "C" {

int oracle_load_lapack(const char* path) {
  void* h = dlopen(path, RTLD_NOW | RTLD_LOCAL);
  if (!h) { g_err = dlerror(); return -1; }
  g_dspev = (dspev_t)dlsym(h, "scipy_dspev_");
  if (!g_dspev) g_dspev = (dspev_t)dlsym(h, "dspev_");
  g_dgemm = (dgemm_t)dlsym(h, "scipy_cblas_dgemm");
  if (!g_dgemm) g_dgemm = (dgemm_t)dlsym(h, "cblas_dgemm");
  g_setthreads = (setthreads_t)dlsym(h, "scipy_openblas_set_num_threads");
  if (!g_setthreads) g_setthreads = (setthreads_t)dlsym(h, "openblas_set_num_threads");
  if (!g_dspev || !g_dgemm) { g_err = "dspev/dgemm symbols not found"; return -2; }
  return 0;
}

const char* oracle_last_error(void) { return g_err.c_str(); }

void oracle_blas_threads(int n) { if (g_setthreads) g_setthreads(n); }

double oracle_cgordan(double j1, double m1, double j2, double m2, double j, double m) {
  return cgordan(j1, m1, j2, m2, j, m);
}

// CNRGmatrix::DiagBlock (NRGmatrixClass.cpp:566-656): dspev('V','L') on the
// row-major packed upper triangle; row k of Z is eigenvector k.
int oracle_diag_block(int n, const double* packed, double* w, double* Z) {
  if (!g_dspev) { g_err = "LAPACK not loaded"; return -1; }
  std::vector<double> A(packed, packed + (size_t)n * (n + 1) / 2), work(3 * (size_t)n);
  int info = 0, ldz = n;
  const char jobz = 'V', uplo = 'L';
  g_dspev(&jobz, &uplo, &n, A.data(), w, Z, &ldz, work.data(), &info, 1, 1);
  return info;
}

void* oracle_run(const oracle_config* cfg) {
  if (!g_dspev) { g_err = "LAPACK not loaded"; return nullptr; }
  auto t0 = std::chrono::steady_clock::now();
  OracleRun* R = new OracleRun();
  Ctx c;
  const double pi = 3.141592653589793238462643383279502884197169;
  double Lambda = cfg->lambda;
  double HLF = 0.5 * (1.0 + 1.0 / Lambda);
  // a caller's chain (chi_N, e_N) replaces SetChainWilson's; the impurity
  // coupling then carries sqrt(A_Lambda) unless chain_alambda is 0
  // (NRG_main.cpp:204-207)
  const bool custom = cfg->chain_len > 0;
  if (custom && cfg->chain_len < cfg->nsites) { g_err = "chain shorter than nsites"; delete R; return nullptr; }
  double ALambda = std::sqrt(0.5 * std::log(Lambda) * (Lambda + 1) / (Lambda - 1));
  if (custom && !cfg->chain_alambda) ALambda = 1.0;
  double eps = cfg->degen_eps > 0 ? cfg->degen_eps : 1.0e-18;
  int nthreads = cfg->nthreads > 0 ? cfg->nthreads : 1;
  // SetChainWilson (NRGchainClass.cpp:132-155).
  auto chin = [&](int N) {
    if (custom) return cfg->chain_chi[N];
    double d0 = 1.0 - std::pow(Lambda, -((double)N + 1.0));
    double d1 = std::sqrt(1.0 - std::pow(Lambda, -(2.0 * (double)N + 1.0)));
    double d2 = std::sqrt(1.0 - std::pow(Lambda, -(2.0 * (double)N + 3.0)));
    return d0 / (d1 * d2);
  };
  auto onsite = [&](int N) { return custom ? cfg->chain_en[N] : 0.0; };
  c.m.kind = cfg->model;
  R->model = cfg->model;
  R->lambda = Lambda;
  const bool dm = cfg->dm != 0;
  if (dm && cfg->model != ORACLE_MODEL_1CHQS && cfg->model != ORACLE_MODEL_2CHQS) {
    g_err = "DM-NRG shells are restated for the |Q S> models only"; delete R; return nullptr;
  }
  // calcdens = 3: the free Wilson chain (ModelNo 3 with ZeroParams,
  // NRGcodehandlerClass.cpp:85-91; CodeHandler_ModelSwitch.cpp:377-420,
  // 667-720, 940-1000).  H_0 is the first site alone and only f_N is kept.
  const bool chain = cfg->chain != 0;
  if (chain && dm) { g_err = "chain and DM-NRG runs are exclusive"; delete R; return nullptr; }
  if (chain && (cfg->model == ORACLE_MODEL_1CHS || cfg->model == ORACLE_MODEL_1CHSZ)) {
    g_err = "the reference has no free-chain run for the superconducting-lead models"; delete R; return nullptr;
  }
  Arr eig;
  std::vector<Mat> mats;
  std::vector<double> P;
  int sq = 1;
  bool totalS = true;
  int nchan = 1;
  double chi1 = std::sqrt(2.0 * cfg->gamma1 / pi) / (std::sqrt(Lambda) * HLF) * ALambda;
  if (chain) {
    // OneChQS_SetChainH0 / OneChQSz_SetChainH0 (Main/Main_SetH0.cpp:3322-3465)
    // are the impurity start-ups' blocks and f elements at U = ed = B = 0.
    const double chi0 = chin(0);
    if (cfg->model == ORACLE_MODEL_1CHQS) {
      c.m.site = site_1chQS(); c.m.totS = {1};
      Mat f; std::vector<Mat> avg;
      hm1_QS(Lambda, HLF, 0.0, 0.0, eig, f, avg);
      mats.push_back(f);
      c.m.op_rule = {R_F_QS}; c.m.op_check = {C_QS_CD};
      P = {Lambda, chi0, 0.0, 0.0};
    } else if (cfg->model == ORACLE_MODEL_1CHQSZ) {
      c.m.site = site_1chQSz(); c.m.totS = {};
      Mat fu, fd; std::vector<Mat> avg;
      hm1_QSz(Lambda, HLF, 0.0, 0.0, 0.0, eig, fu, fd, avg);
      mats.push_back(fu); mats.push_back(fd);
      c.m.op_rule = {R_FUP_QSZ, R_FDN_QSZ}; c.m.op_check = {C_Q_CD, C_Q_CD};
      P = {Lambda, chi0, 0.0, 0.0};
      totalS = false;
    } else if (cfg->model == ORACLE_MODEL_1CHQ) {
      // ModelSwitch has no chain case for OneChQ: NRG_main.cpp:215-218 runs
      // the Anderson model with every parameter zeroed instead (a decoupled
      // impurity, Gamma = 0, from site 0 on; Nsites0 = 0).
      c.m.site = site_1chQ(); c.m.totS = {}; c.m.common = {1, 0, 0};
      Mat fu, fd; std::vector<Mat> avg;
      hm1_Q(Lambda, HLF, 0.0, 0.0, eig, fu, fd, avg);
      mats.push_back(fu); mats.push_back(fd);
      c.m.op_rule = {R_FUP_QSZ, R_FDN_QSZ}; c.m.op_check = {C_Q_CD, C_Q_CD};
      P = {Lambda, 0.0, 0.0, 0.0};
      totalS = false; sq = -1;
    } else if (cfg->model == ORACLE_MODEL_2CHQS) {
      c.m.site = site_2chQS(); c.m.totS = {1};
      Mat f1, f2;
      h0_chain_2chQS(c, eig, f1, f2);
      mats.push_back(f1); mats.push_back(f2);
      c.m.op_rule = {R_F1_2CH, R_F2_2CH}; c.m.op_check = {C_2CH_CD, C_2CH_CD};
      P = {Lambda, chi0, chi0, 0.0, 0.0};
      nchan = 2;
    } else {
      g_err = "unknown model"; delete R; return nullptr;
    }
    eig.nshell = 0;
  } else if (cfg->model == ORACLE_MODEL_1CHQS) {
    c.m.site = site_1chQS(); c.m.totS = {1};
    Mat f; std::vector<Mat> avg;
    hm1_QS(Lambda, HLF, cfg->U, cfg->ed, eig, f, avg);
    if (dm) {
      // calcdens = 1 (CodeHandler_ModelSwitch.cpp:162-176): fN and cdot1, the
      // latter a copy of fN at H_{-1} (Main_SetH0.cpp:1958-1961).
      Mat cd = f; cd.name = "cdot1";
      mats.push_back(f); mats.push_back(cd);
      c.m.op_rule = {R_F_QS, R_CD_QS};
      c.m.op_check = {C_QS_CD, C_QS_CD};
    } else {
      mats.push_back(f); for (auto& x : avg) mats.push_back(x);
      c.m.op_rule = {R_F_QS, R_IMPONLY, R_IMPONLY, R_IMPONLY};
      c.m.op_check = {C_QS_CD, C_DIAG, C_DIAG, C_DIAG};
    }
    P = {Lambda, chi1, 0.0, 0.0};
  } else if (cfg->model == ORACLE_MODEL_1CHQSZ) {
    c.m.site = site_1chQSz(); c.m.totS = {};
    Mat fu, fd; std::vector<Mat> avg;
    hm1_QSz(Lambda, HLF, cfg->U, cfg->ed, cfg->gamma2_or_B, eig, fu, fd, avg);
    mats.push_back(fu); mats.push_back(fd); for (auto& x : avg) mats.push_back(x);
    c.m.op_rule = {R_FUP_QSZ, R_FDN_QSZ, R_IMPONLY, R_IMPONLY};
    c.m.op_check = {C_Q_CD, C_Q_CD, C_DIAG, C_DIAG};
    P = {Lambda, chi1, 0.0, 0.0};
    totalS = false;
  } else if (cfg->model == ORACLE_MODEL_1CHS) {
    // SymNo 7, ModelNo 0, calcdens 0 (CodeHandler_ModelSwitch.cpp:1681-1814):
    // fN (OneChS_fN_MatEl, OneChS_cd_check), n_d, n_d^2, S_d^2 averaged;
    // CommonQNs = {1, 0, 0}, totSpos = {0}; ParamsHN = {Lambda, chi, e_N,
    // Delta_SC} (NRG_main.cpp:264-276).
    c.m.site = site_1chS(); c.m.totS = {0}; c.m.common = {1, 0, 0};
    Mat f; std::vector<Mat> avg;
    hm1_S(Lambda, HLF, cfg->U, cfg->ed, eig, f, avg);
    mats.push_back(f); for (auto& x : avg) mats.push_back(x);
    c.m.op_rule = {R_F_S, R_IMPONLY, R_IMPONLY, R_IMPONLY};
    c.m.op_check = {C_S_CD, C_DIAG, C_DIAG, C_DIAG};
    P = {Lambda, chi1, 0.0, cfg->delta_sc};
    sq = 0;
  } else if (cfg->model == ORACLE_MODEL_1CHSZ) {
    // SymNo 8, ModelNo 0, calcdens 0 (CodeHandler_ModelSwitch.cpp:1825-1970):
    // f_up, f_dn (OneChSz_fN rules and checks), three averaged operators;
    // CommonQNs = {1, 0, 0}, no SU(2); Sqnumber 0.
    c.m.site = site_1chSz(); c.m.totS = {}; c.m.common = {1, 0, 0};
    Mat fu, fd; std::vector<Mat> avg;
    hm1_Sz(Lambda, HLF, cfg->U, cfg->ed, cfg->gamma2_or_B, eig, fu, fd, avg);
    mats.push_back(fu); mats.push_back(fd); for (auto& x : avg) mats.push_back(x);
    c.m.op_rule = {R_FUP_SZ, R_FDN_SZ, R_IMPONLY, R_IMPONLY, R_IMPONLY};
    c.m.op_check = {C_SZ_UP, C_SZ_DN, C_DIAG, C_DIAG, C_DIAG};
    P = {Lambda, chi1, 0.0, cfg->delta_sc};
    totalS = false; sq = 0;
  } else if (cfg->model == ORACLE_MODEL_1CHQ) {
    // SymNo 3 (CodeHandler_ModelSwitch.cpp:1138-1200): f_up, f_dn (OneChQ_fN
    // rules, OneChQ_cd_check), S_z and S_z^2 averaged; CommonQNs = {1, 0, 0}.
    c.m.site = site_1chQ(); c.m.totS = {}; c.m.common = {1, 0, 0};
    Mat fu, fd; std::vector<Mat> avg;
    hm1_Q(Lambda, HLF, cfg->U, cfg->ed, eig, fu, fd, avg);
    mats.push_back(fu); mats.push_back(fd); for (auto& x : avg) mats.push_back(x);
    c.m.op_rule = {R_FUP_QSZ, R_FDN_QSZ, R_IMPONLY, R_IMPONLY};
    c.m.op_check = {C_Q_CD, C_Q_CD, C_DIAG, C_DIAG};
    P = {Lambda, chi1, 0.0, 0.0};
    totalS = false; sq = -1;
  } else if (cfg->model == ORACLE_MODEL_2CHQS) {
    c.m.site = site_2chQS(); c.m.totS = {1};
    Mat f; std::vector<Mat> avg;
    hm1_QS(Lambda, HLF, cfg->U, cfg->ed, eig, f, avg);
    if (dm) {
      // f_N of both channels and c_d, all copies of d at H_{-1}.
      Mat f2 = f, cd = f; cd.name = "cdot1";
      mats.push_back(f); mats.push_back(f2); mats.push_back(cd);
      c.m.op_rule = {R_F1_2CH, R_F2_2CH, R_CD_2CH};
      c.m.op_check = {C_2CH_CD, C_2CH_CD, C_2CH_CD};
    } else {
      mats.push_back(f); mats.push_back(f); for (auto& x : avg) mats.push_back(x);
      c.m.op_rule = {R_F1_2CH, R_F2_2CH, R_IMPONLY, R_IMPONLY, R_IMPONLY};
      c.m.op_check = {C_2CH_CD, C_2CH_CD, C_DIAG, C_DIAG, C_DIAG};
    }
    double chi2 = std::sqrt(2.0 * cfg->gamma2_or_B / pi) / (std::sqrt(Lambda) * HLF) * ALambda;
    P = {Lambda, chi1, chi2, 0.0, 0.0};
    nchan = 2;
  } else {
    g_err = "unknown model"; delete R; return nullptr;
  }
  for (size_t i = 0; i < mats.size(); ++i) {
    if (c.m.op_rule[i] == R_IMPONLY) { mats[i].need_old = true; mats[i].calc_avg = true; }
    else if (c.m.op_rule[i] == R_CD_QS || c.m.op_rule[i] == R_CD_2CH) { mats[i].need_old = true; mats[i].calc_avg = false; }
    else { mats[i].need_old = false; mats[i].calc_avg = false; }
  }
  R->nqn = (cfg->model == ORACLE_MODEL_1CHQ || cfg->model == ORACLE_MODEL_1CHS || cfg->model == ORACLE_MODEL_1CHSZ)
               ? 1 : 2;
  for (auto& m : mats) if (m.calc_avg) R->opnames.push_back(m.name);
  const double betabar = 0.727;
  Basis cut, ab;
  cut_states(eig, cut, cfg->ncutoff, eps);
  for (auto& m : mats) if (m.calc_avg) R->opavg_m1.push_back(calc_opavg(cut, m, betabar, totalS, sq));
  int N0 = 0;
  if (chain && cfg->model != ORACLE_MODEL_1CHQ) {
    // Nsites0 = 1: CalcThermo on H_0 before the loop, at D = HLF
    // Lambda^(-(Nsites0-2)/2) (NRG_main.cpp:242-255).
    OracleIter I;
    I.params = P;
    const double D0 = HLF * std::pow(Lambda, 0.5);
    I.qn = eig.qn;
    for (int b = 0; b < eig.nblocks(); ++b) { I.bsize.push_back(eig.bsize(b)); I.kept_bsize.push_back(eig.bsize(b)); }
    I.en = eig.en;
    I.nkept = eig.nstates();
    for (int nc = 1; nc <= 4; ++nc) {
      double bN = betabar * std::pow(Lambda, (nc - 4) / (2.0 * 4));
      I.thermo.push_back(bN); I.thermo.push_back(D0 / bN);
      I.thermo.push_back(calc_suscep(eig, bN, sq, totalS));
      I.thermo.push_back(calc_entropy(eig, bN, sq, totalS));
    }
    R->it.push_back(std::move(I));
    N0 = 1;
  }
  const int ien = nchan + 1;  // e_N's place in ParamsHN (NRG_main.cpp:272-276)
  for (int N = N0; N < cfg->nsites; ++N) {
    const auto t_iter = std::chrono::steady_clock::now();
    OracleIter I;
    P[ien] = onsite(N);  // GetEn(Nsites) (NRG_main.cpp:198, 408-413)
    I.params = P;
    double DN = HLF * std::pow(Lambda, (-(N - 1) / 2.0));
    build_basis(c.m, cut, ab, dm);
    bool cap = (cfg->capture_iter == N);
    if (cap) {
      I.basis_qn = ab.qn; I.basis_en = ab.en; I.basis_bbe = ab.bbe;
      I.basis_itype = ab.itype; I.basis_stcf = ab.stcf;
      I.capd["old_qn"] = cut.qn; I.capi["old_bbe"] = cut.bbe;
      for (size_t o = 0; o < mats.size(); ++o) {
        I.capi["old_map." + std::to_string(o)] = mats[o].map;
        I.capi["old_mbe." + std::to_string(o)] = mats[o].mbe;
        I.capd["old_el." + std::to_string(o)] = mats[o].el;
      }
      I.capd["basis_qn"] = ab.qn; I.capi["basis_bbe"] = ab.bbe; I.capd["basis_en"] = ab.en;
      I.capi["basis_itype"] = ab.itype; I.capi["basis_stcf"] = ab.stcf;
    }
    std::vector<std::vector<double>> H;
    diag_hn(c, P, ab, mats, eig, nthreads, cap ? &H : nullptr, &I.emin);
    if (cap) for (auto& h : H) I.H.insert(I.H.end(), h.begin(), h.end());
    if (cap) { I.capd["eig_en"] = eig.en; I.capd["eig_evec"] = eig.evec; I.capd["params"] = P; }
    I.ecut = set_kept(eig, cfg->ncutoff, eps, &I.nkept);
    if (cap) { I.capd["kept_en"] = eig.en; I.capi["kept"] = std::vector<int>(eig.kept.begin(), eig.kept.end()); }
    I.qn = eig.qn;
    for (int b = 0; b < eig.nblocks(); ++b) I.bsize.push_back(eig.bsize(b));
    I.en = eig.en;
    for (int nc = 1; nc <= 4; ++nc) {
      double bN = betabar * std::pow(Lambda, (nc - 4) / (2.0 * 4));
      I.thermo.push_back(bN); I.thermo.push_back(DN / bN);
      I.thermo.push_back(calc_suscep(eig, bN, sq, totalS));
      I.thermo.push_back(calc_entropy(eig, bN, sq, totalS));
    }
    if (dm) {
      // UpdateBefCut = 1 (NRG_main.cpp:334-343, 393-396): operators are
      // updated in the uncut basis, then the shell is saved, then the cut.
      Basis full;
      cut_states(eig, full, 2 * eig.nstates(), eps);
      update_matrices(c, full, ab, mats, nthreads);
      DmShell shl;
      shl.ab = ab; shl.full = full; shl.cd = mats.back();
      R->dm.push_back(std::move(shl));
    }
    cut_states(eig, cut, cfg->ncutoff, eps);
    if (cap) {
      I.capd["cut_qn"] = cut.qn; I.capi["cut_bbe"] = cut.bbe; I.capi["cut_bbe_bc"] = cut.bbe_bc;
      I.capi["cut_bbe_eig"] = cut.bbe_eig; I.capi["cut_stcf"] = cut.stcf; I.capd["cut_en"] = cut.en;
      I.capi["cut_kept"] = std::vector<int>(cut.kept.begin(), cut.kept.end()); I.capd["cut_evec"] = cut.evec;
    }
    if (!dm) update_matrices(c, cut, ab, mats, nthreads);
    if (cap)
      for (size_t o = 0; o < mats.size(); ++o) {
        I.capi["new_map." + std::to_string(o)] = mats[o].map;
        I.capi["new_mbe." + std::to_string(o)] = mats[o].mbe;
        I.capd["new_el." + std::to_string(o)] = mats[o].el;
      }
    for (auto& m : mats) if (m.calc_avg) I.opavg.push_back(calc_opavg(cut, m, betabar, totalS, sq));
    for (int b = 0; b < cut.nblocks(); ++b) I.kept_bsize.push_back(cut.bsize(b));
    for (int ich = 0; ich < nchan; ++ich) P[ich + 1] = chin(N);
    // Delta_SC rescaled for the next iteration by CNRGchain::ScaleFactor(N)
    // (NRG_main.cpp:414-419; NRGchainClass.cpp:187-202, z = 1)
    if (cfg->model == ORACLE_MODEL_1CHS || cfg->model == ORACLE_MODEL_1CHSZ)
      P[3] = std::pow(Lambda, 0.5 * (double)N) / HLF * cfg->delta_sc;
    I.seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_iter).count();
    R->it.push_back(std::move(I));
  }
  R->seconds = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  return R;
}

void oracle_free(void* h) { delete (OracleRun*)h; }

int oracle_num_iters(void* h) { return (int)((OracleRun*)h)->it.size(); }
int oracle_nqn(void* h) { return ((OracleRun*)h)->nqn; }
double oracle_seconds(void* h) { return ((OracleRun*)h)->seconds; }
int oracle_num_ops(void* h) { return (int)((OracleRun*)h)->opnames.size(); }
const char* oracle_op_name(void* h, int k) { return ((OracleRun*)h)->opnames[k].c_str(); }
const double* oracle_opavg_m1(void* h) { return ((OracleRun*)h)->opavg_m1.data(); }

#define ITER(h, n) (((OracleRun*)h)->it[n])
int oracle_iter_nblocks(void* h, int n) { return (int)ITER(h, n).bsize.size(); }
const double* oracle_iter_qn(void* h, int n) { return ITER(h, n).qn.data(); }
const int* oracle_iter_bsize(void* h, int n) { return ITER(h, n).bsize.data(); }
int oracle_iter_nstates(void* h, int n) { return (int)ITER(h, n).en.size(); }
const double* oracle_iter_en(void* h, int n) { return ITER(h, n).en.data(); }
double oracle_iter_emin(void* h, int n) { return ITER(h, n).emin; }
double oracle_iter_ecut(void* h, int n) { return ITER(h, n).ecut; }
double oracle_iter_seconds(void* h, int n) { return ITER(h, n).seconds; }
int oracle_iter_nkept(void* h, int n) { return ITER(h, n).nkept; }
const double* oracle_iter_thermo(void* h, int n) { return ITER(h, n).thermo.data(); }
const double* oracle_iter_opavg(void* h, int n) { return ITER(h, n).opavg.data(); }
int oracle_iter_nparams(void* h, int n) { return (int)ITER(h, n).params.size(); }
const double* oracle_iter_params(void* h, int n) { return ITER(h, n).params.data(); }
int oracle_iter_nkeptblocks(void* h, int n) { return (int)ITER(h, n).kept_bsize.size(); }
const int* oracle_iter_kept_bsize(void* h, int n) { return ITER(h, n).kept_bsize.data(); }
int oracle_iter_H_size(void* h, int n) { return (int)ITER(h, n).H.size(); }
const double* oracle_iter_H(void* h, int n) { return ITER(h, n).H.data(); }
const int* oracle_iter_basis_itype(void* h, int n) { return ITER(h, n).basis_itype.data(); }
const int* oracle_iter_basis_stcf(void* h, int n) { return ITER(h, n).basis_stcf.data(); }
const double* oracle_iter_basis_en(void* h, int n) { return ITER(h, n).basis_en.data(); }

// DM-NRG on the shells of a run made with cfg->dm: the backward sweep of the
// density matrix and the FDM spectral function of c_d at the given
// frequencies, or (omegas == NULL) on CalcSpec_ManyOmegas's grid with nw
// points per shell.  Returns the number of frequencies written (at most cap),
// or -1.  rho_trace, if not NULL, receives sum_b (2S_b+1) Tr rho_N(b) per shell.
int oracle_dm_spectral(void* h, const oracle_dm_params* prm, const double* omegas, int nomega, double* omega_out,
                       double* a_out, int cap, double* rho_trace) {
  OracleRun* R = (OracleRun*)h;
  if (R->dm.empty()) { g_err = "run has no DM-NRG shells"; return -1; }
  Ctx c;
  c.m.kind = R->model;
  c.m.site = R->model == ORACLE_MODEL_2CHQS ? site_2chQS() : site_1chQS();
  DmParams p{R->lambda, prm->temp, prm->betabar, prm->bbroad, prm->twindow, prm->broadtemp, prm->site_dim, 0.0};
  dm_temperature(p, (int)R->dm.size(), prm->mtemp, prm->temp);
  std::vector<RhoBlocks> rho;
  dm_backward(c, R->dm, p, rho);
  if (rho_trace)
    for (size_t N = 0; N < rho.size(); ++N) {
      const Arr& a = R->dm[N].full;
      double t = 0.0;
      for (int b = 0; b < a.nblocks(); ++b) {
        int n = a.bsize(b);
        double deg = a.totalS ? 2.0 * a.q(b, a.sqn[0]) + 1.0 : 1.0;
        for (int i = 0; i < n; ++i) t += deg * rho[N][b][(size_t)i * n + i];
      }
      rho_trace[N] = t;
    }
  std::vector<double> om;
  if (omegas) om.assign(omegas, omegas + nomega);
  else spec_grid(R->lambda, (int)R->dm.size(), prm->nw, om);
  int n = std::min<int>((int)om.size(), cap);
  for (int k = 0; k < n; ++k) {
    omega_out[k] = om[k];
    a_out[k] = spec_at(c, R->dm, rho, p, om[k]);
  }
  return n;
}

// One shell's term of the sum over shells: FDM_SpecDens_M_STL(omegabar, N)
// (the last shell: CalcSpecCosti_T_N).
double oracle_dm_shell_term(void* h, const oracle_dm_params* prm, int N, double omegabar) {
  OracleRun* R = (OracleRun*)h;
  if (R->dm.empty() || N < 0 || N >= (int)R->dm.size()) return 0.0;
  Ctx c;
  c.m.kind = R->model;
  c.m.site = R->model == ORACLE_MODEL_2CHQS ? site_2chQS() : site_1chQS();
  DmParams p{R->lambda, prm->temp, prm->betabar, prm->bbroad, prm->twindow, prm->broadtemp, prm->site_dim, 0.0};
  dm_temperature(p, (int)R->dm.size(), prm->mtemp, prm->temp);
  std::vector<RhoBlocks> rho;
  dm_backward(c, R->dm, p, rho);
  return spec_fdm(c, R->dm, rho, N, p, omegabar);
}

// The DM-NRG shells of a run made with cfg->dm, field by field (NULL and
// *len = -1 if absent): basis_qn/bbe/itype/stcf/en (Abasis_N), qn/bbe/en/
// kept/evec (Acut_N), cd_map/cd_mbe/cd_el (c_d).
const double* oracle_dm_d(void* h, int N, const char* name, int* len) {
  OracleRun* R = (OracleRun*)h;
  *len = -1;
  if (N < 0 || N >= (int)R->dm.size()) return nullptr;
  const DmShell& s = R->dm[N];
  const std::string k(name);
  const std::vector<double>* v = nullptr;
  if (k == "basis_qn") v = &s.ab.qn; else if (k == "basis_en") v = &s.ab.en; else if (k == "qn") v = &s.full.qn;
  else if (k == "en") v = &s.full.en; else if (k == "evec") v = &s.full.evec; else if (k == "cd_el") v = &s.cd.el;
  if (!v) return nullptr;
  *len = (int)v->size();
  return v->data();
}
const int* oracle_dm_i(void* h, int N, const char* name, int* len) {
  OracleRun* R = (OracleRun*)h;
  *len = -1;
  if (N < 0 || N >= (int)R->dm.size()) return nullptr;
  static thread_local std::vector<int> kept;
  const DmShell& s = R->dm[N];
  const std::string k(name);
  const std::vector<int>* v = nullptr;
  if (k == "basis_bbe") v = &s.ab.bbe; else if (k == "basis_itype") v = &s.ab.itype;
  else if (k == "basis_stcf") v = &s.ab.stcf; else if (k == "bbe") v = &s.full.bbe;
  else if (k == "cd_map") v = &s.cd.map; else if (k == "cd_mbe") v = &s.cd.mbe;
  else if (k == "kept") { kept.assign(s.full.kept.begin(), s.full.kept.end()); v = &kept; }
  if (!v) return nullptr;
  *len = (int)v->size();
  return v->data();
}

// Named captures of the capture iteration: NULL (and *len = -1) if absent.
const double* oracle_cap_d(void* h, int n, const char* name, int* len) {
  auto& m = ITER(h, n).capd;
  auto it = m.find(name);
  if (it == m.end()) { *len = -1; return nullptr; }
  *len = (int)it->second.size();
  return it->second.data();
}
const int* oracle_cap_i(void* h, int n, const char* name, int* len) {
  auto& m = ITER(h, n).capi;
  auto it = m.find(name);
  if (it == m.end()) { *len = -1; return nullptr; }
  *len = (int)it->second.size();
  return it->second.data();
}

}  // extern "C"
