// Host-side model tables of the GB300 NRG engine (see nrg_model.h).
#include "nrg_model.h"

#include <algorithm>
#include <cmath>
#include <mutex>
#include <stdexcept>

namespace nrg {

namespace {
// dEqual.cpp:6 and :17.
inline bool deq(double a, double b) { return std::fabs(a - b) < 1.e-20; }
inline bool dleq(double a, double b) { return (a < b) || (std::fabs(a - b) < 1.e-20); }

double factorial(int n) {
  if (n < 0) return 0.0;
  unsigned __int128 p = 1;
  for (int k = 2; k <= n; ++k) p *= (unsigned)k;
  return (double)p;  // n! rounded once, as a table of factorials holds it
}

// CGordan.cpp:13.
bool triangle(double J1, double J2, double J) {
  return !((J - (J1 + J2) > 1.0e-10) || (J - std::fabs(J1 - J2) < -1.0e-10));
}

// Single-site operator tables.  OneCh_fd_table (OpTables.cpp:8-33) gives
// <t_i| f^dagger_sigma |t_j> in the basis |0>,|up>,|dn>,|up dn>.
double fd_onech(int sigma, int ti, int tj) {
  if (sigma == 1) return ((ti == 1 && tj == 0) || (ti == 3 && tj == 2)) ? 1.0 : 0.0;
  if (sigma == -1) { if (ti == 2 && tj == 0) return 1.0; if (ti == 3 && tj == 1) return -1.0; }
  return 0.0;
}

// OneChS_fd_table (OpTables.cpp:419-443): <t_i| f^dagger_sigma |t_j> in the
// basis |0>, |up dn>, |up>, |dn> of the superconducting-lead site.
double fd_onechS(int sigma, int ti, int tj) {
  if (sigma == 1) return ((ti == 2 && tj == 0) || (ti == 1 && tj == 3)) ? 1.0 : 0.0;
  if (sigma == -1) { if (ti == 3 && tj == 0) return 1.0; if (ti == 1 && tj == 2) return -1.0; }
  return 0.0;
}

// TwoChQS_fd_table (TwoChQS_OpTables.cpp:20-130): the reference's table of
// f^dagger_{ch,sigma} in the 16-state two-channel site basis.
struct TwoChTables {
  double fd[2][2][16][16];  // [ch-1][sigma==+1][ti][tj]
  double spsm[16][16];      // TwoChQS_SpSm_table (:140-185)
  TwoChTables() {
    for (auto& a : fd) for (auto& b : a) for (auto& c : b) for (double& x : c) x = 0.0;
    const double r = 1.0 / std::sqrt(2.0), mr = -1.0 / std::sqrt(2.0);
    auto& u1 = fd[0][1]; auto& d1 = fd[0][0]; auto& u2 = fd[1][1]; auto& d2 = fd[1][0];
    u1[2][0] = 1; u1[10][1] = 1; u1[9][3] = r; u1[11][6] = 1; u1[5][3] = r;
    u1[7][4] = 1; u1[12][9] = r; u1[12][5] = mr; u1[14][8] = 1; u1[15][13] = 1;
    d1[4][0] = 1; d1[9][1] = r; d1[5][1] = mr; d1[8][3] = 1; d1[13][6] = 1;
    d1[7][2] = -1; d1[12][10] = -1; d1[14][9] = mr; d1[14][5] = mr; d1[15][11] = -1;
    u2[1][0] = 1; u2[6][3] = 1; u2[10][2] = -1; u2[11][9] = mr; u2[11][5] = mr;
    u2[9][4] = mr; u2[5][4] = r; u2[13][8] = -1; u2[12][7] = 1; u2[15][14] = 1;
    d2[3][0] = 1; d2[6][1] = -1; d2[9][2] = mr; d2[11][10] = 1; d2[5][2] = mr;
    d2[8][4] = -1; d2[13][9] = r; d2[13][5] = mr; d2[14][7] = 1; d2[15][12] = -1;
    for (int i = 0; i < 16; ++i) for (int j = 0; j < 16; ++j) spsm[i][j] = (i == j) ? 1.0 : 0.0;
    const int pairs[][2] = {{1, 3}, {2, 4}, {11, 13}, {12, 14}, {8, 9}, {9, 10}, {8, 10}};
    for (auto& p : pairs) { spsm[p[0]][p[1]] = 1.0; spsm[p[1]][p[0]] = 1.0; }
  }
  double f(int ch, int sigma, int ti, int tj) const {
    if (ti < 0 || tj < 0 || ti > 15 || tj > 15 || (ch != 1 && ch != 2) || (sigma != 1 && sigma != -1)) return 0.0;
    return fd[ch - 1][sigma == 1][ti][tj];
  }
};
const TwoChTables& twoch() { static TwoChTables t; return t; }

void site_block(Site& s, std::initializer_list<double> q, int n) {
  std::vector<double> v(q);
  s.blk.push(v.data(), n);
  s.nstates += n;
}
}  // namespace

double clebsch(double J1, double M1, double J2, double M2, double J, double M) {
  if ((J1 < 0.0) || (J2 < 0.0) || (J < 0.0)) return 0.0;
  if ((std::fabs(M1) > J1) || (std::fabs(M2) > J2) || (std::fabs(M) > J)) return 0.0;
  if (std::fabs(M - (M1 + M2)) > 1.0e-10) return 0.0;
  if ((J > (J1 + J2)) || (J < std::fabs(J1 - J2))) return 0.0;
  double a = factorial((int)(J1 + J2 - J)) * factorial((int)(J1 - J2 + J)) * factorial((int)(-J1 + J2 + J)) *
             (2 * J + 1) / factorial((int)(J1 + J2 + J + 1));
  double rho = a > 0.0 ? std::sqrt(a) : 0.0;
  double s = factorial((int)(J + M)) * factorial((int)(J - M)) * factorial((int)(J1 + M1)) *
             factorial((int)(J1 - M1)) * factorial((int)(J2 + M2)) * factorial((int)(J2 - M2));
  double sigma = s > 0.0 ? std::sqrt(s) : 0.0;
  int rmax = std::min(std::min((int)(J1 - M1), (int)(J2 + M2)), (int)(J1 + J2 - J));
  int rmin = std::max(std::max(-(int)(J - J2 + M1), -(int)(J - J1 - M2)), 0);
  double tau = 0.0;
  for (int r = rmin; r <= rmax; r++) {
    double d = factorial((int)(J1 - M1) - r) * factorial((int)(J2 + M2) - r) * factorial((int)(J - J2 + M1) + r) *
               factorial((int)(J - J1 - M2) + r) * factorial((int)(J1 + J2 - J) - r) * factorial(r);
    tau += std::pow(-1.0, r) * (1.0 / d);
  }
  return rho * sigma * tau;
}

namespace {
// Memoised Clebsch-Gordan: pure function of six half-integers.  Shared by
// the host threads of batched sweeps, hence the lock.
double cg(double a, double b, double c, double d, double e, double f) {
  static std::map<std::array<double, 6>, double> memo;
  static std::mutex mu;
  std::array<double, 6> k{a, b, c, d, e, f};
  {
    std::lock_guard<std::mutex> lock(mu);
    auto it = memo.find(k);
    if (it != memo.end()) return it->second;
  }
  double v = clebsch(a, b, c, d, e, f);
  std::lock_guard<std::mutex> lock(mu);
  memo.emplace(k, v);
  return v;
}
}  // namespace

void BlockArray::push(const double* q, int n) {
  for (int k = 0; k < nqn; ++k) qn.push_back(q[k]);
  offset.push_back(nstates());
  size.push_back(n);
}

int BlockArray::find(const double* q) const {
  for (int b = 0; b < nblocks(); ++b) {
    bool ok = true;
    for (int k = 0; k < nqn && ok; ++k) ok = deq(qn[(size_t)b * nqn + k], q[k]);
    if (ok) return b;
  }
  return -1;
}

int Site::block_of_state(int t) const {
  for (int b = 0; b < blk.nblocks(); ++b)
    if (t >= blk.offset[b] && t < blk.offset[b] + blk.size[b]) return b;
  return -1;
}

int OpBlocks::find(int i, int j) const {
  for (size_t k = 0; k < bi.size(); ++k)
    if (bi[k] == i && bj[k] == j) return (int)k;
  return -1;
}

ModelSpec make_model(ModelKind kind) {
  ModelSpec m;
  m.kind = kind;
  if (kind == MODEL_1CHQS) {
    // OneChQS_SetSingleSite (OneChQS_SetSingleSite.cpp:5-44): (Q,S,Sz), one state per block.
    m.site.blk.nqn = 3;
    site_block(m.site, {-1, 0, 0}, 1); site_block(m.site, {0, 0.5, 0.5}, 1);
    site_block(m.site, {0, 0.5, -0.5}, 1); site_block(m.site, {1, 0, 0}, 1);
    m.totalS = true; m.nchan = 1; m.nsigma = 1;
    m.op_kind = {OP_F_QS, OP_IMPONLY, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_QS_CD, CHK_DIAG, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fN", "Ndot", "NdSq", "SdSq"};
  } else if (kind == MODEL_1CHQSZ) {
    // OneChQSz_SetSingleSite (Main/Main_SetSingleSite.cpp:347-380).
    m.site.blk.nqn = 2;
    site_block(m.site, {-1, 0}, 1); site_block(m.site, {0, 0.5}, 1);
    site_block(m.site, {0, -0.5}, 1); site_block(m.site, {1, 0}, 1);
    m.totalS = false; m.nchan = 1; m.nsigma = 2;
    m.op_kind = {OP_FUP_QSZ, OP_FDN_QSZ, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_Q_CD, CHK_Q_CD, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fNup", "fNdn", "Ndot", "Szdot"};
  } else if (kind == MODEL_1CHQ) {
    // CNRGCodeHandler::SetSingleSite, SymNo 3 (NRGcodehandlerClass.cpp:484-503):
    // blocks by Q alone, |0> | |up>,|dn> | |up dn> (types 0..3).
    m.site.blk.nqn = 2;
    site_block(m.site, {-1, 0}, 1); site_block(m.site, {0, 0}, 2); site_block(m.site, {1, 0}, 1);
    m.totalS = false; m.nchan = 1; m.nsigma = 2;
    // CodeHandler_ModelSwitch.cpp:1138-1158: f_up, f_dn, and S_z, S_z^2 averaged.
    m.op_kind = {OP_FUP_QSZ, OP_FDN_QSZ, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_Q_CD, CHK_Q_CD, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fNup", "fNdn", "Sz", "Sz2"};
  } else if (kind == MODEL_1CHS) {
    // CNRGCodeHandler::SetSingleSite, SymNo 7 (NRGcodehandlerClass.cpp:536-560):
    // (S,Sz) blocks |0>,|up dn> | |up> | |dn> (types 0..3), here (0,S,Sz).
    m.site.blk.nqn = 3;
    site_block(m.site, {0, 0, 0}, 2); site_block(m.site, {0, 0.5, 0.5}, 1); site_block(m.site, {0, 0.5, -0.5}, 1);
    m.totalS = true; m.nchan = 1; m.nsigma = 1;
    // CodeHandler_ModelSwitch.cpp:1699-1721 (calcdens 0): fN, and n_d, n_d^2,
    // S_d^2 averaged.
    m.op_kind = {OP_F_S, OP_IMPONLY, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_S_CD, CHK_DIAG, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fN", "Ndot", "NdSq", "SdSq"};
  } else if (kind == MODEL_1CHSZ) {
    // CNRGCodeHandler::SetSingleSite, SymNo 8 (NRGcodehandlerClass.cpp:564-584):
    // Sz blocks |0>,|up dn> | |up> | |dn>, here (0,Sz).
    m.site.blk.nqn = 2;
    site_block(m.site, {0, 0}, 2); site_block(m.site, {0, 0.5}, 1); site_block(m.site, {0, -0.5}, 1);
    m.totalS = false; m.nchan = 1; m.nsigma = 2;
    // CodeHandler_ModelSwitch.cpp:1846-1880 (calcdens 0): f_up, f_dn, and
    // three averaged operators named Ndot, NdSq, SdSq that OneChSz_SetAnderson_Hm1
    // fills with n_d, S_z, S_z^2.
    m.op_kind = {OP_FUP_SZ, OP_FDN_SZ, OP_IMPONLY, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_SZ_UP, CHK_SZ_DN, CHK_DIAG, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fNup", "fNdn", "Ndot", "NdSq", "SdSq"};
  } else if (kind == MODEL_2CHQS) {
    // TwoChQS_SetSingleSite (TwoChQS_SetSingleSite.cpp:5-124): 16 states in 10 blocks.
    m.site.blk.nqn = 3;
    site_block(m.site, {-2, 0, 0}, 1); site_block(m.site, {-1, 0.5, 0.5}, 2);
    site_block(m.site, {-1, 0.5, -0.5}, 2); site_block(m.site, {0, 0, 0}, 3);
    site_block(m.site, {0, 1, -1}, 1); site_block(m.site, {0, 1, 0}, 1);
    site_block(m.site, {0, 1, 1}, 1); site_block(m.site, {1, 0.5, 0.5}, 2);
    site_block(m.site, {1, 0.5, -0.5}, 2); site_block(m.site, {2, 0, 0}, 1);
    m.totalS = true; m.nchan = 2; m.nsigma = 2;
    m.op_kind = {OP_F1_2CH, OP_F2_2CH, OP_IMPONLY, OP_IMPONLY, OP_IMPONLY};
    m.op_check = {CHK_2CH_CD, CHK_2CH_CD, CHK_DIAG, CHK_DIAG, CHK_DIAG};
    m.op_name = {"fNch1", "fNch2", "Ndot", "NdSq", "SdSq"};
  } else {
    throw std::runtime_error("unknown model");
  }
  for (int k : m.op_kind) m.op_avg.push_back(k == OP_IMPONLY ? 1 : 0);
  // Old operators entering H_N and the element arithmetic of the assembly:
  // OneChQ_HN_MatEl is OneChQSz_HN_MatEl without the e_N term (zero on the
  // flat band), the same arithmetic.
  m.nops_h = (kind == MODEL_1CHQS || kind == MODEL_1CHS) ? 1 : 2;
  m.hn_form = kind == MODEL_1CHQ ? (int)MODEL_1CHQSZ : (int)kind;
  m.onsite = kind != MODEL_2CHQS;
  return m;
}

namespace {
void plugin_fail(const char* what) { throw std::invalid_argument(std::string("model description: ") + what); }
}  // namespace

ModelSpec make_plugin_model(const nrg_model_desc& d) {
  if (d.total_spin != 0 && d.total_spin != 1) plugin_fail("total_spin must be 0 or 1");
  if (d.site_nqn != (d.total_spin ? 3 : 2)) plugin_fail("site_nqn must be 3 with total_spin, else 2");
  if (d.site_nblocks < 1 || !d.site_qn || !d.site_bsize) plugin_fail("no site blocks");
  if (d.hn_form < NRG_HN_ONE_OP || d.hn_form > NRG_HN_CHANNEL_SUM) plugin_fail("unknown hn_form");
  if (!d.hn_coef || !d.op_check) plugin_fail("hn_coef and op_check are required");
  const int hn_ops = d.hn_form == NRG_HN_ONE_OP ? 1 : 2;
  if (d.nops < hn_ops || d.nops > 8 || !d.op_class) plugin_fail("nops must cover the operators entering H_N (at most 8)");
  ModelSpec m;
  m.kind = MODEL_PLUGIN;
  m.site.blk.nqn = d.site_nqn;
  for (int b = 0; b < d.site_nblocks; ++b) {
    if (d.site_bsize[b] < 1) plugin_fail("empty site block");
    m.site.blk.push(d.site_qn + (size_t)b * d.site_nqn, d.site_bsize[b]);
    m.site.nstates += d.site_bsize[b];
  }
  m.totalS = d.total_spin == 1;
  m.nchan = d.hn_form == NRG_HN_CHANNEL_SUM ? 2 : 1;
  m.nsigma = d.hn_form == NRG_HN_ONE_OP ? 1 : 2;
  m.nops_h = hn_ops;
  m.hn_form = d.hn_form == NRG_HN_ONE_OP ? (int)MODEL_1CHQS
              : d.hn_form == NRG_HN_SPIN_SUM ? (int)MODEL_1CHQSZ : (int)MODEL_2CHQS;
  m.onsite = d.onsite != 0;
  for (int o = 0; o < d.nops; ++o) {
    const int cls = d.op_class[o];
    if (cls == NRG_OP_SITE) m.op_kind.push_back(OP_PLUGIN_SITE + o);
    else if (cls == NRG_OP_IMPURITY) m.op_kind.push_back(OP_PLUGIN_IMP + o);
    else if (cls == NRG_OP_IMPURITY_DIAG) m.op_kind.push_back(OP_IMPONLY);
    else plugin_fail("unknown op_class");
    if (cls != NRG_OP_IMPURITY_DIAG && !d.op_factor) plugin_fail("op_factor is required");
    m.op_check.push_back(CHK_PLUGIN + o);
    m.op_name.push_back("op" + std::to_string(o));
    m.op_avg.push_back(d.op_avg && d.op_avg[o] ? 1 : 0);
  }
  m.ext = &d;
  m.cache = std::make_shared<PluginCache>();
  return m;
}

StartState make_plugin_start(const ModelSpec& m) {
  const nrg_model_desc& d = *m.ext;
  if (d.start_nblocks < 1 || !d.start_qn || !d.start_bsize || !d.start_en || !d.start_npairs)
    plugin_fail("no H_{-1} blocks");
  StartState s;
  s.blk.nqn = 2;
  for (int b = 0; b < d.start_nblocks; ++b) {
    if (d.start_bsize[b] < 1) plugin_fail("empty H_{-1} block");
    s.blk.push(d.start_qn + 2 * (size_t)b, d.start_bsize[b]);
  }
  s.en.assign(d.start_en, d.start_en + s.blk.nstates());
  for (double e : s.en)
    if (!std::isfinite(e)) plugin_fail("non-finite H_{-1} level");
  size_t pr = 0;
  int64_t el = 0;
  for (int o = 0; o < d.nops; ++o) {
    OpBlocks ob;
    if (d.start_npairs[o] < 0) plugin_fail("negative pair count");
    if (d.start_npairs[o] > 0 && (!d.start_pairs || !d.start_el)) plugin_fail("missing H_{-1} operator blocks");
    for (int k = 0; k < d.start_npairs[o]; ++k, ++pr) {
      const int i = d.start_pairs[2 * pr], j = d.start_pairs[2 * pr + 1];
      if (i < 0 || j < 0 || i >= d.start_nblocks || j >= d.start_nblocks) plugin_fail("H_{-1} operator block out of range");
      const int64_t n = (int64_t)d.start_bsize[i] * d.start_bsize[j];
      ob.bi.push_back(i); ob.bj.push_back(j); ob.off.push_back((int64_t)ob.el.size());
      for (int64_t x = 0; x < n; ++x) {
        const double v = d.start_el[el + x];
        if (!std::isfinite(v)) plugin_fail("non-finite H_{-1} operator element");
        ob.el.push_back(v);
      }
      el += n;
    }
    s.ops.push_back(std::move(ob));
  }
  return s;
}

namespace {
void diag_op(const BlockArray& a, const std::vector<double>& v, OpBlocks& o) {
  for (int b = 0; b < a.nblocks(); ++b) {
    o.bi.push_back(b); o.bj.push_back(b); o.off.push_back((int64_t)o.el.size()); o.el.push_back(v[b]);
  }
}
void single(OpBlocks& o, int i, int j, double v) {
  o.bi.push_back(i); o.bj.push_back(j); o.off.push_back((int64_t)o.el.size()); o.el.push_back(v);
}
}  // namespace

StartState make_start(const ModelSpec& m, double lambda, double U, double ed, double B) {
  StartState s;
  double HLF = 0.5 * (1.0 + 1.0 / lambda);
  double scale = lambda * HLF;
  s.blk.nqn = 2;
  if (m.kind == MODEL_1CHQS || m.kind == MODEL_2CHQS) {
    // OneChQS_SetAnderson_Hm1 (Main/Main_SetH0.cpp:1794-1969): the impurity
    // multiplets |0>, |sigma>, |up dn> in units of Lambda*HLF, reduced
    // <||d||> = (1, -sqrt 2), and n_d, n_d^2, S^2 on the diagonal.
    const double q[3][2] = {{-1, 0}, {0, 0.5}, {1, 0}};
    for (auto& x : q) s.blk.push(x, 1);
    s.en = {0.5 * U / scale, (ed + 0.5 * U) / scale, (2.0 * ed + 1.5 * U) / scale};
    OpBlocks f;
    single(f, 0, 1, 1.0);
    single(f, 1, 2, -std::sqrt(2.0));
    std::vector<double> nd, nd2, s2;
    for (int b = 0; b < 3; ++b) {
      double n = s.blk.q(b, 0) + 1.0, S = s.blk.q(b, 1);
      nd.push_back(n); nd2.push_back(n * n); s2.push_back(S * (S + 1.0));
    }
    OpBlocks o1, o2, o3;
    diag_op(s.blk, nd, o1); diag_op(s.blk, nd2, o2); diag_op(s.blk, s2, o3);
    s.ops.push_back(f);
    if (m.kind == MODEL_2CHQS) s.ops.push_back(f);  // f_ch1 = f_ch2 = d
    s.ops.push_back(o1); s.ops.push_back(o2); s.ops.push_back(o3);
  } else if (m.kind == MODEL_1CHS) {
    // OneChS_SetAnderson_Hm1 (Main/Main_SetH0.cpp:2618-2738): blocks S = 0
    // (|0>, |up dn>) and S = 1/2; reduced <||f||> between them; n_d, n_d^2,
    // S^2 diagonal.
    const double q[2][2] = {{0, 0}, {0, 0.5}};
    s.blk.push(q[0], 2); s.blk.push(q[1], 1);
    s.en = {0.5 * U / scale, (2.0 * ed + 1.5 * U) / scale, (ed + 0.5 * U) / scale};
    OpBlocks f, nd, nd2, s2;
    auto pair = [](OpBlocks& o, int i, int j, std::initializer_list<double> v) {
      o.bi.push_back(i); o.bj.push_back(j); o.off.push_back((int64_t)o.el.size());
      o.el.insert(o.el.end(), v);
    };
    pair(f, 0, 1, {1.0, 0.0}); pair(f, 1, 0, {0.0, -std::sqrt(2.0)});
    pair(nd, 0, 0, {0.0, 0.0, 0.0, 2.0}); pair(nd, 1, 1, {1.0});
    pair(nd2, 0, 0, {0.0, 0.0, 0.0, 4.0}); pair(nd2, 1, 1, {1.0});
    pair(s2, 0, 0, {0.0, 0.0, 0.0, 0.0}); pair(s2, 1, 1, {0.75});
    s.ops = {f, nd, nd2, s2};
  } else if (m.kind == MODEL_1CHSZ) {
    // OneChSz_SetAnderson_Hm1 (Main/Main_SetH0.cpp:2751-2933): Sz blocks 0
    // (|0>, |up dn>), +1/2, -1/2 with the Zeeman term -hz S_z, hz = B/2;
    // f_up, f_dn not reduced; n_d, S_z, S_z^2 diagonal.
    const double hz = 0.5 * B;
    const double q[3][2] = {{0, 0}, {0, 0.5}, {0, -0.5}};
    s.blk.push(q[0], 2); s.blk.push(q[1], 1); s.blk.push(q[2], 1);
    s.en = {0.5 * U / scale, (2.0 * ed + 1.5 * U) / scale, (ed + 0.5 * U - hz) / scale, (ed + 0.5 * U + hz) / scale};
    OpBlocks fu, fd, nd, sz, sz2;
    auto pair = [](OpBlocks& o, int i, int j, std::initializer_list<double> v) {
      o.bi.push_back(i); o.bj.push_back(j); o.off.push_back((int64_t)o.el.size());
      o.el.insert(o.el.end(), v);
    };
    pair(fu, 0, 1, {1.0, 0.0}); pair(fu, 2, 0, {0.0, 1.0});
    pair(fd, 0, 2, {1.0, 0.0}); pair(fd, 1, 0, {0.0, -1.0});
    pair(nd, 0, 0, {0.0, 0.0, 0.0, 2.0}); pair(nd, 1, 1, {1.0}); pair(nd, 2, 2, {1.0});
    pair(sz, 0, 0, {0.0, 0.0, 0.0, 0.0}); pair(sz, 1, 1, {0.5}); pair(sz, 2, 2, {-0.5});
    pair(sz2, 0, 0, {0.0, 0.0, 0.0, 0.0}); pair(sz2, 1, 1, {0.25}); pair(sz2, 2, 2, {0.25});
    s.ops = {fu, fd, nd, sz, sz2};
  } else if (m.kind == MODEL_1CHQ) {
    // OneChQ_SetAnderson_Hm1 (Main/Main_SetH0.cpp:217-352): |0> | |up>,|dn> |
    // |up dn> by Q, the Q = 0 block two-fold; f_up, f_dn not reduced; S_z and
    // S_z^2 from the states' iDegen/10.
    const double q[3][2] = {{-1, 0}, {0, 0}, {1, 0}};
    s.blk.push(q[0], 1); s.blk.push(q[1], 2); s.blk.push(q[2], 1);
    s.en = {0.5 * U / scale, (ed + 0.5 * U) / scale, (ed + 0.5 * U) / scale, (2.0 * ed + 1.5 * U) / scale};
    OpBlocks fu, fd, sz, sz2;
    auto pair = [](OpBlocks& o, int i, int j, std::initializer_list<double> v) {
      o.bi.push_back(i); o.bj.push_back(j); o.off.push_back((int64_t)o.el.size());
      o.el.insert(o.el.end(), v);
    };
    pair(fu, 0, 1, {1.0, 0.0}); pair(fu, 1, 2, {0.0, 1.0});
    pair(fd, 0, 1, {0.0, 1.0}); pair(fd, 1, 2, {-1.0, 0.0});
    pair(sz, 0, 0, {0.0}); pair(sz, 1, 1, {0.5, 0.0, 0.0, -0.5}); pair(sz, 2, 2, {0.0});
    pair(sz2, 0, 0, {0.0}); pair(sz2, 1, 1, {0.25, 0.0, 0.0, 0.25}); pair(sz2, 2, 2, {0.0});
    s.ops = {fu, fd, sz, sz2};
  } else {
    // OneChQSz_SetAnderson_Hm1 (Main/Main_SetH0.cpp:421-660) with the Zeeman
    // term -hz S_z, hz = B/2.
    double hz = 0.5 * B;
    const double q[4][2] = {{-1, 0}, {0, 0.5}, {0, -0.5}, {1, 0}};
    for (auto& x : q) s.blk.push(x, 1);
    s.en = {0.5 * U / scale, (ed + 0.5 * U - hz) / scale, (ed + 0.5 * U + hz) / scale, (2.0 * ed + 1.5 * U) / scale};
    OpBlocks fu, fd, nd, sz;
    single(fu, 0, 1, 1.0); single(fu, 2, 3, 1.0);
    single(fd, 0, 2, 1.0); single(fd, 1, 3, -1.0);
    std::vector<double> vn, vs;
    for (int b = 0; b < 4; ++b) { vn.push_back(s.blk.q(b, 0) + 1.0); vs.push_back(s.blk.q(b, 1)); }
    diag_op(s.blk, vn, nd); diag_op(s.blk, vs, sz);
    s.ops = {fu, fd, nd, sz};
  }
  return s;
}

StartState make_chain_start(const ModelSpec& m, double lambda) {
  const int nf = m.kind == MODEL_1CHQS ? 1 : 2;  // f_N operators entering H_N
  if (m.kind != MODEL_2CHQS) {
    // OneChQS_SetChainH0 / OneChQSz_SetChainH0 (Main/Main_SetH0.cpp:3322-3465):
    // the site multiplets at zero energy carry the same blocks and reduced f
    // elements as the impurity start with U = ed = B = 0.
    StartState s = make_start(m, lambda, 0.0, 0.0, 0.0);
    s.ops.resize(nf);
    return s;
  }
  // TwoChQS_SetH0Chain (Main/Main_SetH0.cpp:3472-3560): the two-channel site
  // in its multiplet basis -- the highest-weight state (Sz = S) of every site
  // block, blocks in order of first appearance, all from one "old" state --
  // and f_ch = SetMatrix over that basis with the rule UpdateMatrices uses.
  BlockArray vac;
  vac.nqn = 2;
  const double q0[2] = {0.0, 0.0};
  vac.push(q0, 1);
  Basis B;
  build_basis(m, vac, B);
  StartState s;
  s.blk = B.blk;
  s.en.assign(B.blk.nstates(), 0.0);
  for (int o = 0; o < nf; ++o) {
    OpBlocks f;
    for (int i = 0; i < B.blk.nblocks(); ++i)
      for (int j = 0; j < B.blk.nblocks(); ++j) {
        if (!op_check(m, m.op_check[o], B.blk, i, j)) continue;
        f.bi.push_back(i); f.bj.push_back(j); f.off.push_back((int64_t)f.el.size());
        for (int a = B.blk.offset[i]; a < B.blk.offset[i] + B.blk.size[i]; ++a)
          for (int b = B.blk.offset[j]; b < B.blk.offset[j] + B.blk.size[j]; ++b)
            f.el.push_back(op_site_factor(m, m.op_kind[o], B.blk.q(i, 1), B.blk.q(j, 1), B.itype[a], B.itype[b]));
      }
    s.ops.push_back(f);
  }
  return s;
}

void build_basis(const ModelSpec& m, const BlockArray& kept, Basis& out) {
  // BuildBasis (BuildBasis.cpp:8-432) with CommonQNs = {2, 0,1, 0,1} and,
  // for SU(2) models, totSpos = {1}.
  const BlockArray& ss = m.site.blk;
  out = Basis();
  out.blk.nqn = 2;
  std::vector<double> cand;
  for (int b = 0; b < kept.nblocks(); ++b) {
    double Qo = kept.q(b, 0), So = kept.q(b, 1);
    for (int s = 0; s < ss.nblocks(); ++s) {
      double Qs = ss.q(s, 0), Ss = ss.q(s, 1);
      cand.push_back(Qs + Qo); cand.push_back(Ss + So);
      if (m.totalS) {
        for (double Sn = So + Ss - 1.0; Sn >= std::fabs(So - Ss); Sn -= 1.0) {
          cand.push_back(Qs + Qo); cand.push_back(Sn);
        }
      }
    }
  }
  // FilterQNumbers (NRGarrayClass.cpp:271-309): keep first occurrences.
  std::vector<double> qn;
  for (size_t k = 0; k < cand.size(); k += 2) {
    bool dup = false;
    for (size_t j = 0; j < qn.size() && !dup; j += 2) dup = (qn[j] == cand[k] && qn[j + 1] == cand[k + 1]);
    if (!dup) { qn.push_back(cand[k]); qn.push_back(cand[k + 1]); }
  }
  int nb = (int)qn.size() / 2;
  out.seg.resize(nb);
  for (int b = 0; b < nb; ++b) {
    double Qn = qn[2 * b], Sn = qn[2 * b + 1];
    int local = 0;
    for (int bo = 0; bo < kept.nblocks(); ++bo) {
      double Qo = kept.q(bo, 0), So = kept.q(bo, 1);
      for (int s = 0; s < ss.nblocks(); ++s) {
        bool ok = deq(Qn, ss.q(s, 0) + Qo);
        if (m.totalS) ok = ok && deq(Sn, ss.q(s, 2) + So) && triangle(So, ss.q(s, 1), Sn);
        else ok = ok && deq(Sn, ss.q(s, 1) + So);
        if (!ok) continue;
        Segment g{bo, s, local, kept.size[bo], ss.size[s]};
        int sidx = (int)out.seg[b].size();
        out.seg[b].push_back(g);
        for (int a = 0; a < g.count; ++a)
          for (int u = 0; u < g.nsite; ++u) {
            out.itype.push_back(ss.offset[s] + u);
            out.stcf.push_back(kept.offset[bo] + a);
            out.seg_of.push_back(sidx);
            out.a_of.push_back(a);
          }
        local += g.count * g.nsite;
      }
    }
    out.blk.push(&qn[2 * b], local);
  }
}

namespace {
// Coefficient of OneChQS_HN_MatEl (OpMatRules.cpp:1473-1523) for the site
// pair (typep, type) in a new multiplet of spin Si, times the fermion sign.
double hn_coef_1chQS(const Site& st, double Si, int typep, int type) {
  const BlockArray& ss = st.blk;
  double Qtp = ss.q(typep, 0), Stp = ss.q(typep, 1), Sztp = ss.q(typep, 2);
  double Qt = ss.q(type, 0), Stt = ss.q(type, 1), Szt = ss.q(type, 2);
  double Scfp = Si - Sztp, Scf = Si - Szt;
  double fermi = deq(Qt, 0.0) ? -1.0 : 1.0;
  double coef = 0.0;
  double qp[3] = {Qtp, Stp, Sztp}, qq[3] = {Qt, Stt, Szt};
  for (double Sz = -Stt; Sz <= Stt; Sz += 1.0) {
    qq[2] = Sz;
    int sst = ss.find(qq);
    for (int sigma = -1; sigma <= 1; sigma += 2) {
      double dS = 0.5 * (double)sigma;
      double Szcf = Si - Sz, Szcfp = Szcf - dS, Szp = Sz + dS;
      qp[2] = Sz + dS;
      int sstp = ss.find(qp);
      double a0 = cg(Scf, Szcf, Stt, Sz, Si, Si);
      double a1 = cg(Scfp, Szcfp, Stp, Szp, Si, Si);
      double a2 = cg(Scfp, Szcfp, 0.5, dS, Scf, Szcf);
      double a3 = fd_onech(sigma, sstp, sst);
      coef += a0 * a1 * a2 * a3;
    }
  }
  return coef * fermi;  // fermi = +-1: multiplying first or last is exact
}

// Per-(channel, sigma) sum FullMatEl of TwoChQS_HN_MatEl
// (TwoChQS_OpMatRules.cpp:843-957) for the site pair (typep, type).
double hn_full_2chQS(const Site& st, double Si, int typep, int type, int ich, int sigma) {
  const BlockArray& ss = st.blk;
  const TwoChTables& T = twoch();
  int bp = st.block_of_state(typep), b = st.block_of_state(type);
  double Stp = ss.q(bp, 1), Sztp = ss.q(bp, 2), Stt = ss.q(b, 1), Szt = ss.q(b, 2);
  double Soldp = Si - Sztp, Sold = Si - Szt;
  double fermi = (deq(Szt, 0.5) || deq(Szt, -0.5)) ? -1.0 : 1.0;
  double qp[3] = {ss.q(bp, 0), ss.q(bp, 1), ss.q(bp, 2)}, qq[3] = {ss.q(b, 0), ss.q(b, 1), ss.q(b, 2)};
  double dS = 0.5 * (double)sigma;
  double full = 0.0;
  for (double Szold = Sold; Szold >= -Sold; Szold -= 1.0) {
    double Szoldp = Szold - dS, Sz = Si - Szold, Szp = Sz + dS;
    qp[2] = Szp; qq[2] = Sz;
    int sbp = ss.find(qp), sb = ss.find(qq);
    if (!(dleq(std::fabs(Szp), Stp) && dleq(std::fabs(Szold), Sold) && dleq(std::fabs(Szoldp), Soldp))) continue;
    double a0 = cg(Sold, Szold, Stt, Sz, Si, Si);
    double a1 = cg(Soldp, Szoldp, Stp, Szp, Si, Si);
    double a2 = cg(Soldp, Szoldp, 0.5, dS, Sold, Szold);
    // GetBlockLimit of a missing block (-1) is state 0 (NRGarrayClass.cpp:335).
    int p0 = sbp < 0 ? 0 : ss.offset[sbp], p1 = sbp < 0 ? 0 : ss.offset[sbp] + ss.size[sbp] - 1;
    int s0 = sb < 0 ? 0 : ss.offset[sb], s1 = sb < 0 ? 0 : ss.offset[sb] + ss.size[sb] - 1;
    for (int sp = p0; sp <= p1; sp++)
      for (int s = s0; s <= s1; s++) {
        double x0 = T.spsm[s][type], x1 = T.spsm[sp][typep];
        double a3 = T.f(ich, sigma, sp, s);
        full += a0 * a1 * a2 * a3 * fermi * x0 * x1;
      }
  }
  return full;
}
}  // namespace

// Hopping coefficient of OneChS_HNsc_MatEl (OpMatRules.cpp:1846-1998) for
// the site pair (typep, type) in a new multiplet of spin Si, times its
// fermion sign.  A spin-1/2 site state is looked up as (its site block) + 1,
// which is its type, and as type 0 when no block has the wanted (S, Sz) --
// the reference's lookup, kept.
double hn_coef_1chS(const Site& st, double Si, int typep, int type) {
  const BlockArray& ss = st.blk;
  auto q = [&](int t, int k) { return ss.q(st.block_of_state(t), k); };
  auto lookup = [&](double S, double Sz) { const double x[3] = {0.0, S, Sz}; return ss.find(x) + 1; };
  const double Stildep = q(typep, 1), Sztp0 = q(typep, 2);
  const double Stilde = q(type, 1), Szt0 = q(type, 2);
  const double Scfp = Si - Sztp0, Scf = Si - Szt0;
  const double fermi = (type == 2 || type == 3) ? -1.0 : 1.0;
  double coef = 0.0;
  for (double Sztilde = -Stilde; Sztilde <= Stilde; Sztilde += 1.0) {
    int sitestate = type;
    if (type == 2 || type == 3) sitestate = lookup(Stilde, Sztilde);
    for (int sigma = -1; sigma <= 1; sigma += 2) {
      const double dS = 0.5 * (double)sigma;
      const double Szcf = Si - Sztilde, Szcfp = Szcf - dS, Sztildep = Sztilde + dS;
      int sitestatep = lookup(Stildep, Sztildep);
      if (deq(Sztildep, 0.0)) sitestatep = typep;
      const double a0 = cg(Scf, Szcf, Stilde, Sztilde, Si, Si);
      const double a1 = cg(Scfp, Szcfp, Stildep, Sztildep, Si, Si);
      const double a2 = cg(Scfp, Szcfp, 0.5, dS, Scf, Szcf);
      const double a3 = fd_onechS(sigma, sitestatep, sitestate);
      coef += a0 * a1 * a2 * a3;
    }
  }
  return coef * fermi;  // fermi = +-1: multiplying here or after chi*old is exact
}

void build_hn_tables(const ModelSpec& m, const Basis& b, HNTables& t) {
  int NT = m.site.nstates;
  t.ntypes = NT; t.nchan = m.nchan; t.nsigma = m.nsigma;
  size_t pb = t.per_block();
  t.coef.assign(pb * b.blk.nblocks(), 0.0);
  std::map<double, size_t> done;  // tables depend on the block's S (or Sz) only
  for (int blk = 0; blk < b.blk.nblocks(); ++blk) {
    double Si = b.blk.q(blk, 1);
    double* c = &t.coef[pb * blk];
    auto it = done.find(Si);
    if (it != done.end()) { std::copy(t.coef.begin() + it->second, t.coef.begin() + it->second + pb, c); continue; }
    done.emplace(Si, pb * blk);
    for (int ti = 0; ti < NT; ++ti)
      for (int tj = 0; tj < NT; ++tj) {
        size_t base = ((size_t)ti * NT + tj) * t.nchan * t.nsigma;
        if (m.kind == MODEL_PLUGIN) {
          for (int ch = 0; ch < t.nchan; ++ch)
            for (int s = 0; s < t.nsigma; ++s)
              for (int dir = 0; dir < 2; ++dir) {
                const double v = m.ext->hn_coef(m.ext->user, Si, ti, tj, ch, s, dir);
                if (!std::isfinite(v)) plugin_fail("hn_coef returned a non-finite value");
                c[(base + (size_t)ch * t.nsigma + s) * 2 + dir] = v;
              }
        } else if (m.kind == MODEL_1CHQS) {
          c[base * 2 + 0] = hn_coef_1chQS(m.site, Si, ti, tj);
          c[base * 2 + 1] = hn_coef_1chQS(m.site, Si, tj, ti);
        } else if (m.kind == MODEL_1CHS) {
          c[base * 2 + 0] = hn_coef_1chS(m.site, Si, ti, tj);
          c[base * 2 + 1] = hn_coef_1chS(m.site, Si, tj, ti);
        } else if (m.kind == MODEL_1CHSZ) {
          // OneChSz_HNsc_MatEl (OpMatRules.cpp:2160-2200): per spin, the fermion
          // sign of the "type" state (types 2, 3 carry one electron) times
          // <typep|f^dagger_sigma|type>.
          for (int s = 0; s < 2; ++s) {
            const int isigma = s == 0 ? 1 : -1;
            const double fj = (tj == 2 || tj == 3) ? -1.0 : 1.0, fi = (ti == 2 || ti == 3) ? -1.0 : 1.0;
            c[(base + s) * 2 + 0] = fj * fd_onechS(isigma, ti, tj);
            c[(base + s) * 2 + 1] = fi * fd_onechS(isigma, tj, ti);
          }
        } else if (m.kind == MODEL_1CHQSZ || m.kind == MODEL_1CHQ) {
          // OneChQSz_HN_MatEl (OpMatRules.cpp:468-531), OneChQ_HN_MatEl
          // (:1065-1147): per spin, the fermion sign of the "type" state times
          // <typep|f^dagger_sigma|type>.
          for (int s = 0; s < 2; ++s) {
            int isigma = s == 0 ? 1 : -1;
            double fq = deq(m.site.blk.q(m.site.block_of_state(tj), 0), 0.0) ? -1.0 : 1.0;
            double bq = deq(m.site.blk.q(m.site.block_of_state(ti), 0), 0.0) ? -1.0 : 1.0;
            c[(base + s) * 2 + 0] = fq * fd_onech(isigma, ti, tj);
            c[(base + s) * 2 + 1] = bq * fd_onech(isigma, tj, ti);
          }
        } else {
          for (int ch = 0; ch < 2; ++ch)
            for (int s = 0; s < 2; ++s) {
              int sigma = s == 0 ? -1 : 1;
              size_t k = base + (size_t)ch * 2 + s;
              c[k * 2 + 0] = hn_full_2chQS(m.site, Si, ti, tj, ch + 1, sigma);
              c[k * 2 + 1] = hn_full_2chQS(m.site, Si, tj, ti, ch + 1, sigma);
            }
        }
      }
  }
}

double sc_pair_1chS(int ti, int tj) { return (ti == 1 && tj == 0) ? 1.0 : 0.0; }
bool hc_switch_1chS(int ti, int tj) { return fd_onechS(1, ti, tj) == 0.0 && fd_onechS(-1, ti, tj) == 0.0; }
bool hc_switch_1chSz(int sigma, int ti, int tj) { return fd_onechS(sigma, ti, tj) == 0.0; }

double op_site_factor(const ModelSpec& m, int op, double Si, double Sj, int ti, int tj) {
  const BlockArray& ss = m.site.blk;
  if (op >= OP_PLUGIN_SITE) {
    const int o = op >= OP_PLUGIN_IMP ? op - OP_PLUGIN_IMP : op - OP_PLUGIN_SITE;
    const auto key = std::make_tuple(o, Si, Sj, ti, tj);
    auto it = m.cache->factor.find(key);
    if (it != m.cache->factor.end()) return it->second;
    const double v = m.ext->op_factor(m.ext->user, o, Si, Sj, ti, tj);
    if (!std::isfinite(v)) plugin_fail("op_factor returned a non-finite value");
    m.cache->factor.emplace(key, v);
    return v;
  }
  if (op == OP_F_S) {
    // OneChS_fN_MatEl (OpMatRules.cpp:1555-1654), with its site lookups.
    auto q = [&](int t, int k) { return ss.q(m.site.block_of_state(t), k); };
    auto lookup = [&](double S, double Sz) { const double x[3] = {0.0, S, Sz}; return ss.find(x) + 1; };
    const double Stildei = q(ti, 1), Stildej = q(tj, 1);
    const double Scfi = Si - q(ti, 2), Scfj = Sj - q(tj, 2);
    const double sigma = Sj - Si;
    double aux = 0.0, cg1 = 0.0;
    for (double Sztj = -Stildej; Sztj <= Stildej; Sztj += 1.0) {
      int ssj = tj, ssi = ti;
      if (tj == 2 || tj == 3) ssj = lookup(Stildej, Sztj);
      if (ti == 2 || ti == 3) ssi = lookup(Stildei, Sztj - sigma);
      const double cg0 = cg(Scfi, Si - Sztj + sigma, Stildei, Sztj - sigma, Si, Si);
      cg1 = cg(Scfj, Sj - Sztj, Stildej, Sztj, Sj, Sj);
      aux += fd_onechS((int)(sigma / 0.5), ssj, ssi) * cg0 * cg1;
    }
    const double n0 = cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (!deq(n0, 0.0)) return aux / n0;
    if (!deq(cg1, 0.0)) return 0.0 / cg1;
    return 0.0;
  }
  if (op == OP_FUP_SZ) return fd_onechS(1, tj, ti);   // OneChSz_fN_MatEl (OpMatRules.cpp:1986-2014)
  if (op == OP_FDN_SZ) return fd_onechS(-1, tj, ti);
  if (op == OP_FUP_QSZ) return fd_onech(1, tj, ti);   // OneChQ_fN_MatEl (OpMatRules.cpp:1003-1033)
  if (op == OP_FDN_QSZ) return fd_onech(-1, tj, ti);
  if (op == OP_IMPONLY) return ti == tj ? 1.0 : 0.0;
  if (op == OP_CD_QS) {
    // OneChQS_cd_MatEl (OpMatRules.cpp:1249-1330): the impurity d operator
    // recoupled with a site state it leaves unchanged.  A site state that is
    // not found matches another one that is not found, as in the reference.
    double qi[3] = {ss.q(ti, 0), ss.q(ti, 1), ss.q(ti, 2)}, qj[3] = {ss.q(tj, 0), ss.q(tj, 1), ss.q(tj, 2)};
    const double Sti = qi[1], Stj = qj[1];
    const double Scfi = Si - qi[2], Scfj = Sj - qj[2];
    const double fermi = deq(qj[0], 0.0) ? -1.0 : 1.0;
    double sigma = Sj - Si;
    double norm = cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (deq(norm, 0.0)) {
      sigma = Si - Sj;
      norm = cg(Si, Si, 0.5, sigma, Sj, Sj);
      if (deq(norm, 0.0)) return 0.0;
    }
    double f = 0.0;
    for (double Szcfj = -Scfj; Szcfj <= Scfj; Szcfj += 1.0) {
      const double Szcfi = Szcfj - sigma;
      qj[2] = Sj - Szcfj; const int sj = ss.find(qj);
      qi[2] = Si - Szcfi; const int si = ss.find(qi);
      const double a0 = cg(Scfi, Szcfi, Sti, qi[2], Si, Si);
      const double a1 = cg(Scfj, Szcfj, Stj, qj[2], Sj, Sj);
      const double a2 = cg(Scfi, Szcfi, 0.5, sigma, Scfj, Szcfj);
      if (si == sj) f += a0 * a1 * a2 * fermi;
    }
    return f / norm;
  }
  if (op == OP_CD_2CH) {
    // The impurity d operator across the 16-state two-channel site.  The
    // reference has no such rule (TwoChQS keeps no c_d); this is
    // OneChQS_cd_MatEl's recoupling with the site multiplet left unchanged:
    // t_i and t_j are members of one multiplet (TwoChQS_SpSm_table), the
    // site member is the same on both sides, and the Fermi sign is (-1) to
    // the site's fermion number Q + 2, as Q = 0 (one fermion) is for the
    // one-channel site.
    const TwoChTables& T = twoch();
    if (T.spsm[ti][tj] == 0.0) return 0.0;
    const int bi = m.site.block_of_state(ti), bj = m.site.block_of_state(tj);
    const double Qt = ss.q(bi, 0), St = ss.q(bi, 1);
    const double Scfi = Si - ss.q(bi, 2), Scfj = Sj - ss.q(bj, 2);
    const double fermi = std::fabs(std::fmod(Qt, 2.0)) == 1.0 ? -1.0 : 1.0;
    double sigma = Sj - Si;
    double norm = cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (deq(norm, 0.0)) {
      sigma = Si - Sj;
      norm = cg(Si, Si, 0.5, sigma, Sj, Sj);
      if (deq(norm, 0.0)) return 0.0;
    }
    double f = 0.0;
    for (double Szcfj = -Scfj; Szcfj <= Scfj; Szcfj += 1.0) {
      const double Szcfi = Szcfj - sigma;
      const double Sztj = Sj - Szcfj, Szti = Si - Szcfi;
      if (!deq(Szti, Sztj) || std::fabs(Sztj) > St + 1.0e-12) continue;
      const double a0 = cg(Scfi, Szcfi, St, Szti, Si, Si);
      const double a1 = cg(Scfj, Szcfj, St, Sztj, Sj, Sj);
      const double a2 = cg(Scfi, Szcfi, 0.5, sigma, Scfj, Szcfj);
      f += a0 * a1 * a2 * fermi;
    }
    return f / norm;
  }
  if (op == OP_F_QS) {
    // OneChQS_fN_MatEl (OpMatRules.cpp:1167-1244).
    double qi[3] = {ss.q(ti, 0), ss.q(ti, 1), ss.q(ti, 2)}, qj[3] = {ss.q(tj, 0), ss.q(tj, 1), ss.q(tj, 2)};
    double Sti = qi[1], Szti = qi[2], Stj = qj[1], Sztj = qj[2];
    double Scfi = Si - Szti, Scfj = Sj - Sztj;
    double acc = 0.0, c1 = 0.0;
    double sigma = Sj - Si;
    for (double Sz = -Stj; Sz <= Stj; Sz += 1.0) {
      qj[2] = Sz; int sj = ss.find(qj);
      qi[2] = Sz - sigma; int si = ss.find(qi);
      double c0 = cg(Scfi, Si - Sz + sigma, Sti, Sz - sigma, Si, Si);
      c1 = cg(Scfj, Sj - Sz, Stj, Sz, Sj, Sj);
      acc += fd_onech((int)(sigma / 0.5), sj, si) * c0 * c1;
    }
    double n0 = cg(Si, Si, 0.5, sigma, Sj, Sj);
    if (!deq(n0, 0.0)) return acc / n0;
    return 0.0;
  }
  if (op == OP_F1_2CH || op == OP_F2_2CH) {
    // TwoChQS_fN_MatEl (TwoChQS_OpMatRules.cpp:1205-1352).
    int ich = op == OP_F1_2CH ? 1 : 2;
    const TwoChTables& T = twoch();
    int bi = m.site.block_of_state(ti), bj = m.site.block_of_state(tj);
    double qi[3] = {ss.q(bi, 0), ss.q(bi, 1), ss.q(bi, 2)}, qj[3] = {ss.q(bj, 0), ss.q(bj, 1), ss.q(bj, 2)};
    double Scfi = Si - qi[2], Scfj = Sj - qj[2];
    double c0 = cg(Si, Si, 0.5, -0.5, Sj, Sj), c1 = cg(Si, Si, 0.5, 0.5, Sj, Sj);
    int sigma = 0; double norm = 1.0;
    if (!deq(c0, 0.0)) { sigma = -1; norm = c0; }
    else if (!deq(c1, 0.0)) { sigma = 1; norm = c1; }
    if (sigma == 0) return 0.0;
    double acc = 0.0;
    for (double Szcfj = Scfj; Szcfj >= -Scfj; Szcfj -= 1.0) {
      double Szi = Si - Szcfj, Szj = Sj - Szcfj;
      qi[2] = Szi; int bsi = ss.find(qi);
      qj[2] = Szj; int bsj = ss.find(qj);
      double a0 = cg(Scfi, Szcfj, ss.q(bi, 1), Szi, Si, Si);
      double a1 = cg(Scfj, Szcfj, ss.q(bj, 1), Szj, Sj, Sj);
      int i0 = bsi < 0 ? 0 : ss.offset[bsi], i1 = bsi < 0 ? 0 : ss.offset[bsi] + ss.size[bsi] - 1;
      int j0 = bsj < 0 ? 0 : ss.offset[bsj], j1 = bsj < 0 ? 0 : ss.offset[bsj] + ss.size[bsj] - 1;
      for (int si = i0; si <= i1; si++)
        for (int sj = j0; sj <= j1; sj++)
          acc += T.f(ich, sigma, sj, si) * a0 * a1 * T.spsm[si][ti] * T.spsm[sj][tj];
    }
    return acc / norm;
  }
  return 0.0;
}

bool op_check(const ModelSpec& m, int chk, const BlockArray& a, int i, int j) {
  if (chk >= CHK_PLUGIN) {
    const int o = chk - CHK_PLUGIN;
    const auto key = std::make_tuple(o, a.q(i, 0), a.q(i, 1), a.q(j, 0), a.q(j, 1));
    auto it = m.cache->check.find(key);
    if (it != m.cache->check.end()) return it->second;
    const double qi[2] = {a.q(i, 0), a.q(i, 1)}, qj[2] = {a.q(j, 0), a.q(j, 1)};
    const bool v = m.ext->op_check(m.ext->user, o, qi, qj) != 0;
    m.cache->check.emplace(key, v);
    return v;
  }
  // OneChS_cd_check (OpMatRules.cpp:172, S in the second slot here),
  // Diag_check (OpMatRules.cpp:12), OneChQS_cd_check (:106), OneChQ_cd_check
  // (:92), TwoChQS_cd_check (TwoChQS_OpMatRules.cpp:16).
  switch (chk) {
    case CHK_DIAG: return i == j;
    case CHK_S_CD: return deq(a.q(j, 1), a.q(i, 1) + 0.5) || deq(a.q(j, 1), a.q(i, 1) - 0.5);
    case CHK_SZ_UP: return deq(a.q(j, 1), a.q(i, 1) + 0.5);  // OneChSz_cdup_check :188
    case CHK_SZ_DN: return deq(a.q(j, 1), a.q(i, 1) - 0.5);  // OneChSz_cddn_check :199
    case CHK_Q_CD: return deq(a.q(j, 0), a.q(i, 0) + 1.0);
    case CHK_QS_CD:
    case CHK_2CH_CD:
      return deq(a.q(j, 0), a.q(i, 0) + 1.0) && (deq(a.q(j, 1), a.q(i, 1) + 0.5) || deq(a.q(j, 1), a.q(i, 1) - 0.5));
  }
  return false;
}

}  // namespace nrg
