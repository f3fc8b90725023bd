// Host-side model description for the GB300 NRG engine: single-site tables,
// impurity start-up (H_{-1}), basis construction and the coefficient tables
// that let the device assemble H_N and update operators block by block.
//
// The arithmetic of every coefficient follows the reference rule it cites, in
// the same evaluation order, so that the device-assembled Hamiltonian equals
// the reference's element by element.
#pragma once

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <tuple>
#include <vector>

#include "../../include/twochnrg_gb300.h"

namespace nrg {

// MODEL_1CHQ (SymNo 3) conserves the charge only; its blocks carry the
// reference's single quantum number Q plus a constant 0 in the second slot,
// which leaves BuildBasis's block and state order unchanged.
//
// MODEL_1CHS (SymNo 7, superconducting leads) conserves the total spin only;
// its blocks carry a constant 0 in the charge slot and S in the second, so
// that every SU(2) rule reads S where it does for (Q,S).
// MODEL_1CHSZ (SymNo 8) is its |Sz> form with a Zeeman field: blocks (0, Sz).
// MODEL_PLUGIN: a model described by the caller (nrg_model_desc).
enum ModelKind { MODEL_1CHQS = 0, MODEL_1CHQSZ = 1, MODEL_2CHQS = 2, MODEL_1CHQ = 3, MODEL_1CHS = 4, MODEL_1CHSZ = 5,
                 MODEL_PLUGIN = 6 };

// Operator rule ids (how the operator acts on a new site; see build_op_terms).
enum OpKind {
  OP_F_QS = 1,      // OneChQS_fN_MatEl      (OpMatRules.cpp:1167)
  OP_FUP_QSZ = 2,   // OneChQ_fNup_MatEl     (OpMatRules.cpp:1037)
  OP_FDN_QSZ = 3,   // OneChQ_fNdn_MatEl     (OpMatRules.cpp:1046)
  OP_F1_2CH = 4,    // TwoChQS_fNch1_MatEl   (TwoChQS_OpMatRules.cpp:1355)
  OP_F2_2CH = 5,    // TwoChQS_fNch2_MatEl   (TwoChQS_OpMatRules.cpp:1362)
  OP_IMPONLY = 6,   // ImpOnly_MatEl x old   (OpMatRules.cpp:265)
  OP_CD_QS = 7,     // OneChQS_cd_MatEl x old (OpMatRules.cpp:1249)
  OP_F_S = 8,       // OneChS_fN_MatEl       (OpMatRules.cpp:1555)
  OP_FUP_SZ = 9,    // OneChSz_fNup_MatEl    (OpMatRules.cpp:2016)
  OP_FDN_SZ = 10,   // OneChSz_fNdn_MatEl    (OpMatRules.cpp:2027)
  OP_CD_2CH = 11,   // c_d across the two-channel site x old (OneChQS_cd_MatEl's recoupling)
  // Plug-in operators: OP_PLUGIN_SITE + o acts on the new site (like f_N),
  // OP_PLUGIN_IMP + o is an old operator recoupled across the site (like
  // c_d); the factor is the caller's op_factor for operator o.
  OP_PLUGIN_SITE = 1000,
  OP_PLUGIN_IMP = 2000,
};
// CheckForMatEl rule ids.
// CHK_PLUGIN + o: the caller's op_check for operator o.
enum CheckKind { CHK_DIAG = 1, CHK_QS_CD = 2, CHK_Q_CD = 3, CHK_2CH_CD = 4, CHK_S_CD = 5, CHK_SZ_UP = 6,
                 CHK_SZ_DN = 7, CHK_PLUGIN = 1000 };

// Block-structured array: the common part of CNRGarray / CNRGbasisarray
// (include/NRGclasses.hpp:47-349).
struct BlockArray {
  int nqn = 2;
  std::vector<double> qn;       // nblocks * nqn
  std::vector<int> size;        // states per block
  std::vector<int> offset;      // first state of each block
  int nblocks() const { return (int)size.size(); }
  int nstates() const { return offset.empty() ? 0 : offset.back() + size.back(); }
  double q(int b, int k) const { return qn[(size_t)b * nqn + k]; }
  void push(const double* q, int n);
  int find(const double* q) const;  // GetBlockFromQNumbers semantics, -1 if absent
};

// One single-site basis: blocks by (Q,S,Sz) or (Q,Sz); each state has a type.
struct Site {
  BlockArray blk;               // blocks of the site
  int nstates = 0;
  int block_of_state(int t) const;
};

// A contiguous run of new-basis states that share one old kept block and one
// site block (BuildBasis.cpp:292-403 order: old state major, site state minor).
struct Segment {
  int old_block;   // index in the previous kept array
  int site_block;  // index in Site::blk
  int offset;      // first state inside the new block
  int count;       // kept states of the old block
  int nsite;       // states in the site block (stride)
};

// New basis (CNRGbasisarray after BuildBasis).
struct Basis {
  BlockArray blk;
  std::vector<std::vector<Segment>> seg;  // per new block
  // Per state, over all blocks (global state index):
  std::vector<int> itype;     // iType
  std::vector<int> stcf;      // StCameFrom (old kept state, global)
  std::vector<int> seg_of;    // segment index inside its block
  std::vector<int> a_of;      // old state index inside the old block
};

// Callback results of a plug-in model, memoised for one sweep (the
// callbacks are pure functions of their arguments).
struct PluginCache {
  std::map<std::tuple<int, double, double, int, int>, double> factor;
  std::map<std::tuple<int, double, double, double, double>, bool> check;
};

struct ModelSpec {
  ModelKind kind;
  Site site;
  bool totalS;           // SU(2) multiplet basis
  int nchan;             // Wilson channels
  int nsigma;            // spin components summed in H_N (QSz: 2)
  int nops_h = 1;        // old operators entering H_N (the first ones)
  int hn_form = 0;       // element arithmetic of the assembly (AssembleArgs::model)
  bool onsite = true;    // the diagonal adds e_N (Q_site + 1)
  std::vector<int> op_kind, op_check;
  std::vector<std::string> op_name;
  std::vector<char> op_avg;  // CalcAvg operators
  const nrg_model_desc* ext = nullptr;  // MODEL_PLUGIN: the caller's description
  std::shared_ptr<PluginCache> cache;
};

ModelSpec make_model(ModelKind kind);
// A caller-described model (nrg_model_desc): checked, its site basis and
// operator rules taken over.  Throws std::invalid_argument on a malformed
// description.
ModelSpec make_plugin_model(const nrg_model_desc& d);

// Initial impurity data (H_{-1}): kept array with energies and operators in
// dense per-block-pair form (reference MatBlockMap order).
struct OpBlocks {
  std::vector<int> bi, bj;         // block pairs
  std::vector<int64_t> off;        // offset of each pair in el
  std::vector<double> el;          // row-major blocks, concatenated
  int find(int i, int j) const;
};
struct StartState {
  BlockArray blk;
  std::vector<double> en;
  std::vector<OpBlocks> ops;
};
StartState make_start(const ModelSpec& m, double lambda, double U, double ed, double B);
// H_{-1} of a plug-in model, from its description.
StartState make_plugin_start(const ModelSpec& m);
// Free-chain start-up (calcdens = 3, CodeHandler_ModelSwitch.cpp:377-420,
// 667-720, 940-1000): the first Wilson site alone at zero energy (flat band,
// e_0 = 0) with only the channel operators f_N that enter H_N.
StartState make_chain_start(const ModelSpec& m, double lambda);

// BuildBasis (BuildBasis.cpp:8-432) from a kept array.
void build_basis(const ModelSpec& m, const BlockArray& kept, Basis& out);

// One .bin snapshot in the reference's SaveBin layout (binfile.cpp): the
// CNRGarray fields, the CNRGbasisarray ones (kind 1) or the CNRGmatrix ones
// (kind 2).
struct BinShellFile {
  int nshell = 0, nqn = 0;
  bool totalS = false;
  std::vector<double> qn, en, evec, mat_el;
  std::vector<int> bbe, sqnumbers, itype, stcf, bbe_bc, bbe_eig, map, mbe;
  std::vector<unsigned char> kept;
};
bool read_bin_file(const std::string& path, int kind, BinShellFile& f, std::string& err);
std::string bin_path(const char* dir, const char* what, const char* name, int n);

// Coefficient tables for H_N assembly, per new block:
//   coef[((ti*NT + tj)*nchan*nsigma + ch*nsigma + s)*2 + dir]
// dir 0: the old operator is read as (stcf_i, stcf_j); dir 1: as (stcf_j,
// stcf_i) after the reference's zero test.
struct HNTables {
  int ntypes, nchan, nsigma;
  std::vector<double> coef;  // nblocks * ntypes^2 * nchan * nsigma * 2
  size_t per_block() const { return (size_t)ntypes * ntypes * nchan * nsigma * 2; }
};
void build_hn_tables(const ModelSpec& m, const Basis& b, HNTables& t);

// Site factor of an operator between two new-basis states, g(S_i, S_j, t_i,
// t_j): for f-type operators the states came from the same old state; for
// impurity operators (OP_IMPONLY, OP_CD_QS, OP_CD_2CH) g multiplies the old operator
// element between the states they came from.
double op_site_factor(const ModelSpec& m, int op, double Si, double Sj, int ti, int tj);

// Superconducting-lead |S> model (OneChS_HNsc_MatEl, OpMatRules.cpp:1794-2003):
// the pairing table <t_i| f^dagger_up f^dagger_dn |t_j> (OneChS_fdupfddn_table,
// OpTables.cpp:447-462), and whether the hopping term reads the old operator
// as (stcf_j, stcf_i) whatever its (stcf_i, stcf_j) element (both
// OneChS_fd_table(+-1, t_i, t_j) vanish).
double sc_pair_1chS(int ti, int tj);
bool hc_switch_1chS(int ti, int tj);
// |Sz> form (OneChSz_HNsc_MatEl, OpMatRules.cpp:2098-2205): per spin sigma,
// the old operator is read backwards also when OneChS_fd_table(sigma, t_i,
// t_j) vanishes.
bool hc_switch_1chSz(int sigma, int ti, int tj);
bool op_check(const ModelSpec& m, int chk, const BlockArray& kept, int i, int j);

// Clebsch-Gordan <J1 M1; J2 M2 | J M>  (CGordan.cpp:34-120).
double clebsch(double J1, double M1, double J2, double M2, double J, double M);

}  // namespace nrg
